// o3d_output.cu -- the output-cadence writer of write_all_data and
// write_xdmf (src/visualization.f90:242-354), asynchronous.
//
// At every nfre-th step the reference writes ux, uy, uz, pp, |curl u|, the
// Q-criterion, and phi (with a scalar) and nu_t (with LES) as raw FP64
// column-major files outputs/<name>_<num>.bin (stream access, no record
// markers) and an XDMF file outputs/output_<num>.xdmf that describes them for
// ParaView, then goes on with the next step.  Here the fields are first
// gathered on the device into an FP64 snapshot (one kernel and a few copies
// on the context's stream); the device -> host copies of the snapshot run on
// a separate copy stream into pinned memory, and a host thread writes the
// files once they have landed.  The steps that follow run on the context's
// stream meanwhile: they may overwrite every field, not the snapshot.  The
// next output, o3d_output_wait or o3d_destroy waits for the writer first.
#include <cstdio>
#include <string>
#include <thread>

#include "o3d_internal.cuh"
#include "o3d_kernels.h"
#include "o3d_output.h"

namespace o3d {

struct OutWriter {
  double* snap = nullptr;   // device snapshot, cap fields of n doubles
  double* host = nullptr;   // pinned host copy of it
  long long n = 0;
  int cap = 0;
  cudaStream_t cs = nullptr;    // copy stream
  cudaEvent_t ready = nullptr;  // the snapshot is complete (context stream)
  cudaEvent_t landed = nullptr; // the host copy is complete (copy stream)
  std::thread th;
  int status = O3D_OK;          // result of the last writer thread
  std::string err;
};

static void release(OutWriter* w) {
  if (w->snap) cudaFree(w->snap);
  if (w->host) cudaFreeHost(w->host);
  w->snap = nullptr;
  w->host = nullptr;
  w->cap = 0;
}

int out_wait(OutWriter* w) {
  if (!w) return O3D_OK;
  if (w->th.joinable()) w->th.join();
  const int st = w->status;
  if (st != O3D_OK) set_error("%s", w->err.c_str());
  w->status = O3D_OK;
  w->err.clear();
  return st;
}

void out_destroy(OutWriter* w) {
  if (!w) return;
  if (w->th.joinable()) w->th.join();
  release(w);
  if (w->ready) cudaEventDestroy(w->ready);
  if (w->landed) cudaEventDestroy(w->landed);
  if (w->cs) cudaStreamDestroy(w->cs);
  delete w;
}

int out_prepare(OutWriter** pw, long long n, int nfields, double** snap) {
  OutWriter* w = *pw;
  if (!w) {
    w = new OutWriter();
    *pw = w;
    if (cudaStreamCreateWithFlags(&w->cs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->landed, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      set_error("output writer: stream or event creation failed");
      return O3D_ERR_CUDA;
    }
  }
  // the previous output must be on disk before its buffers are reused
  const int st = out_wait(w);
  if (st) return st;
  if (w->n != n || w->cap < nfields) {
    release(w);
    const size_t bytes = (size_t)n * nfields * sizeof(double);
    if (cudaMalloc((void**)&w->snap, bytes) != cudaSuccess) {
      cudaGetLastError();
      set_error("output writer: cudaMalloc of %zu bytes failed", bytes);
      return O3D_ERR_NOMEM;
    }
    if (cudaMallocHost((void**)&w->host, bytes) != cudaSuccess) {
      cudaGetLastError();
      release(w);
      set_error("output writer: cudaMallocHost of %zu bytes failed", bytes);
      return O3D_ERR_NOMEM;
    }
    w->n = n;
    w->cap = nfields;
  }
  *snap = w->snap;
  return O3D_OK;
}

// write_data_item (src/visualization.f90:343-354)
static void data_item(FILE* f, const char* name, int num, int nx, int ny, int nz) {
  fprintf(f, "<Attribute Name=\"%s\" Center=\"Node\">\n", name);
  fprintf(f,
          "<DataItem Format=\"Binary\" DataType=\"Float\" Precision=\"8\" Endian=\"little\" Seek=\"0\" "
          "Dimensions=\"%5d%5d%5d\">\n",
          nz, ny, nx);
  fprintf(f, "%s_%d.bin\n", name, num);
  fprintf(f, "</DataItem>\n");
  fprintf(f, "</Attribute>\n");
}

// write_xdmf (src/visualization.f90:276-341): the same lines and number
// formats (I5 dimensions, F25.12 reals)
static bool write_xdmf(const OutRequest& r, const char* const* names, int nf) {
  const std::string path = r.dir + "/output_" + std::to_string(r.num) + ".xdmf";
  FILE* f = fopen(path.c_str(), "w");
  if (!f) return false;
  fprintf(f, "<?xml version=\"1.0\" ?>\n");
  fprintf(f, "<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" []>\n");
  fprintf(f, "<Xdmf xmlns:xi=\"http://www.w3.org/2001/XInclude\" Version=\"2.0\">\n");
  fprintf(f, "<Domain>\n");
  fprintf(f, "<Topology name=\"topo\" TopologyType=\"3DRectMesh\" Dimensions=\"%5d%5d%5d\"/>\n", r.nz, r.ny, r.nx);
  fprintf(f, "<Geometry name=\"geo\" GeometryType=\"ORIGIN_DXDYDZ\">\n");
  fprintf(f, "<DataItem Dimensions=\"3\" Format=\"XML\">\n");
  fprintf(f, "%25.12f%25.12f%25.12f\n", r.x0, r.y0, r.z0);
  fprintf(f, "</DataItem>\n");
  fprintf(f, "<DataItem Dimensions=\"3\" Format=\"XML\">\n");
  fprintf(f, "%25.12f%25.12f%25.12f\n", r.dx, r.dy, r.dz);
  fprintf(f, "</DataItem>\n");
  fprintf(f, "</Geometry>\n");
  fprintf(f, "<Grid Name=\"%d\" GridType=\"Uniform\">\n", r.num);
  fprintf(f, "<Time Value=\"%25.12f\"/>\n", r.time);
  fprintf(f, "<Topology Reference=\"/Xdmf/Domain/Topology[1]\"/>\n");
  fprintf(f, "<Geometry Reference=\"/Xdmf/Domain/Geometry[1]\"/>\n");
  for (int q = 0; q < nf; ++q) data_item(f, names[q], r.num, r.nx, r.ny, r.nz);
  fprintf(f, "</Grid>\n");
  fprintf(f, "</Domain>\n");
  fprintf(f, "</Xdmf>\n");
  return fclose(f) == 0;
}

int out_submit(OutWriter* w, const OutRequest& r, const char* const* names, int nf, cudaStream_t compute) {
  cudaError_t e = cudaEventRecord(w->ready, compute);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(w->cs, w->ready, 0);
  const size_t fb = (size_t)w->n * sizeof(double);
  for (int q = 0; q < nf && e == cudaSuccess; ++q)
    e = cudaMemcpyAsync(w->host + (size_t)q * w->n, w->snap + (size_t)q * w->n, fb, cudaMemcpyDeviceToHost, w->cs);
  if (e == cudaSuccess) e = cudaEventRecord(w->landed, w->cs);
  if (e != cudaSuccess) {
    set_error("output writer: %s", cudaGetErrorString(e));
    return O3D_ERR_CUDA;
  }
  std::vector<std::string> nm(names, names + nf);
  w->th = std::thread([w, r, nm]() {
    const cudaError_t ce = cudaEventSynchronize(w->landed);
    if (ce != cudaSuccess) {
      w->status = O3D_ERR_CUDA;
      w->err = std::string("output writer: ") + cudaGetErrorString(ce);
      return;
    }
    for (size_t q = 0; q < nm.size(); ++q) {
      const std::string path = r.dir + "/" + nm[q] + "_" + std::to_string(r.num) + ".bin";
      FILE* f = fopen(path.c_str(), "wb");
      const size_t put = f ? fwrite(w->host + q * (size_t)w->n, sizeof(double), (size_t)w->n, f) : 0;
      const bool closed = f && fclose(f) == 0;
      const bool ok = closed && put == (size_t)w->n;
      if (!ok) {
        w->status = O3D_ERR_BADARG;
        w->err = "output writer: cannot write " + path;
        return;
      }
    }
    std::vector<const char*> cn;
    for (auto& s : nm) cn.push_back(s.c_str());
    if (!write_xdmf(r, cn.data(), (int)cn.size())) {
      w->status = O3D_ERR_BADARG;
      w->err = "output writer: cannot write " + r.dir + "/output_" + std::to_string(r.num) + ".xdmf";
    }
  });
  return O3D_OK;
}

}  // namespace o3d
