"""Extract the reference's published statistics rows into small fixtures.

Reads the two TGV statistics series shipped with osinco3d
(examples/tgv_re1600_dns/tgv_stats_re1600_dns.dat and
examples/tgv_re2500_les/tgv_stats_re2500_les.dat, 17 columns written by
write_statistics, src/IOfunctions.f90:552-555) from a checkout of the
reference and keeps the first rows of each as text fixtures.  The fixtures
are committed; this script only needs the reference tree to regenerate them:

    python tests/golden/make_golden.py /path/to/osinco3d
"""
import os
import sys

ROWS = {
    "tgv_re1600_dns": ("examples/tgv_re1600_dns/tgv_stats_re1600_dns.dat", 8),
    "tgv_re2500_les": ("examples/tgv_re2500_les/tgv_stats_re2500_les.dat", 8),
}


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


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <checkout of osinco3d>")
    main(sys.argv[1])
