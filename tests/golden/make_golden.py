"""Extract the reference's published statistics rows into small fixtures.

Reads the two TGV statistics series shipped with osinco3d
(examples/tgv_re1600_dns/tgv_stats_re1600_dns.dat and
examples/tgv_re2500_les/tgv_stats_re2500_les.dat, 17 columns written by
write_statistics, src/IOfunctions.f90:552-555) from a checkout of the
reference and keeps the first rows of each as text fixtures, plus the first
eight columns (t, E_k, eps, eps2, dzeta, <u^2>, <v^2>, <w^2>) of every row
up to t = 10.5 (Re 1600 DNS, past the dissipation peak at t = 8.96) and
t = 5 (Re 2500 LES, 400 rows) for the whole-run series comparisons.  The
fixtures are committed; this script only needs the reference tree to
regenerate them:

    python tests/golden/make_golden.py /path/to/osinco3d
"""
import os
import sys

ROWS = {
    "tgv_re1600_dns": ("examples/tgv_re1600_dns/tgv_stats_re1600_dns.dat", 8),
    "tgv_re2500_les": ("examples/tgv_re2500_les/tgv_stats_re2500_les.dat", 8),
}
SERIES = {"tgv_re1600_dns": 10.5, "tgv_re2500_les": 5.0}
SERIES_COLS = 8


def main(root: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    for name, (rel, nrows) in ROWS.items():
        with open(os.path.join(root, rel)) as fh:
            data = [ln for ln in fh if ln.strip() and not ln.startswith("#")]
        out = os.path.join(here, f"{name}_stats_head.txt")
        with open(out, "w") as fh:
            fh.write(f"# first {nrows} rows of {rel} (osinco3d), 17 columns:\n")
            fh.write("# t E_k eps eps2 dzeta <u2> <v2> <w2> <(dui/dxj)^2> x9\n")
            fh.writelines(data[:nrows])
        print("wrote", out)
        tmax = SERIES[name]
        out = os.path.join(here, f"{name}_series.txt")
        with open(out, "w") as fh:
            fh.write(f"# rows of {rel} (osinco3d) with t <= {tmax}, first {SERIES_COLS} columns:\n")
            fh.write("# t E_k eps eps2 dzeta <u2> <v2> <w2>\n")
            for ln in data:
                cols = ln.split()
                if float(cols[0]) > tmax:
                    break
                fh.write(" ".join(cols[:SERIES_COLS]) + "\n")
        print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <checkout of osinco3d>")
    main(sys.argv[1])
