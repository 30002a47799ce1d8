// lbdem_download_nodes_noalloc: read back the populations and masses of a
// range of nodes without allocating device memory.
//
// Who needs it: a caller that cannot allocate device memory when it reads
// the lattice, e.g. a monitor that samples a few lattice rows every step
// while the run holds nearly all of HBM. lbdem_download_lattice stages the
// whole lattice through a temporary of (19 + 1) doubles per node (3.4 GB for
// a 256x320x256 lattice) taken with cudaMalloc, and cudaMalloc/cudaFree also
// synchronise the whole device. This entry point stages through a fixed
// buffer compiled into the library instead; it calls no cudaMalloc, cudaFree
// or allocating library routine.
//
// The buffer is one per device and shared by every context on that device:
// calls that overlap in time on one device (from two host threads or two
// contexts) race on it and must be serialised by the caller. Its device
// address is looked up (cudaGetSymbolAddress) by the first call on each
// device, which also loads this module's device code if that has not
// happened yet; make that first call before any stream capture. Each call
// makes the context's device current for its own duration.
//
// The call waits for the context's stream but does not read the run's
// device error bits, so it returns the nodes also after a step reported a
// fault (where lbdem_sync and lbdem_download_lattice return that fault).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "lattice_common.cuh"

using namespace lbdem;

namespace {

constexpr long long kMaxNodes = LBDEM_NOALLOC_MAX_NODES;
constexpr int kMaxDevices = 64;

// [19][count] populations followed by [count] masses of one call. Nothing
// here has to start at zero: the kernel writes every element the call
// copies back.
static __device__ __align__(256) double g_nodeStage[(Q + 1) * kMaxNodes];

std::mutex g_stageMutex;
double* g_stageAddr[kMaxDevices] = {};

int fail(lbdem_ctx* ctx, int code, const std::string& msg) {
  ctx->err = msg;
  return code;
}

// Device address of g_nodeStage on ctx's device, looked up once per device
// with that device current.
int stageAddress(lbdem_ctx* ctx, double** out) {
  const int dev = ctx->device;
  if (dev < 0 || dev >= kMaxDevices)
    return fail(ctx, LBDEM_ERR_INVALID, "device ordinal out of range for the staging buffer");
  std::lock_guard<std::mutex> lock(g_stageMutex);
  if (!g_stageAddr[dev]) {
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e == cudaSuccess && prev != dev) e = cudaSetDevice(dev);
    void* p = nullptr;
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_nodeStage);
    if (prev != dev) cudaSetDevice(prev);
    if (e != cudaSuccess)
      return fail(ctx, LBDEM_ERR_CUDA,
                  std::string("cudaGetSymbolAddress(staging buffer): ") + cudaGetErrorString(e));
    g_stageAddr[dev] = (double*)p;
  }
  *out = g_stageAddr[dev];
  return LBDEM_OK;
}

// Same values as exportLattice, for nodes first .. first+count-1 only.
__global__ void exportNodeRange(Consts k, const uint8_t* mask, const void* f, const double* mass,
                                const float* nF, long long first, int count, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const long long x = first + i;
    const int t = mask[x] & TYPE_MASK;
    const bool act = isActiveT(t);
    for (int j = 0; j < Q; ++j) out[(long long)j * count + i] = act ? fget(k, f, j, x) : 0.0;
    out[(long long)Q * count + i] = (k.mixed && t == 0 && k.freeSurface) ? (double)nF[x] : mass[x];
  }
}

}  // namespace

extern "C" int lbdem_download_nodes_noalloc(lbdem_ctx* ctx, int64_t first, int64_t count,
                                            double* f, double* mass) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  if (count > kMaxNodes)
    return fail(ctx, LBDEM_ERR_INVALID,
                "lbdem_download_nodes_noalloc: count " + std::to_string(count) +
                    " exceeds the staging buffer (LBDEM_NOALLOC_MAX_NODES = " +
                    std::to_string(kMaxNodes) + " nodes)");
  if (first < 0 || count < 0 || first > ctx->k.N - count)
    return fail(ctx, LBDEM_ERR_INVALID,
                "lbdem_download_nodes_noalloc: node range [" + std::to_string(first) + ", " +
                    std::to_string(first + count) + ") is outside the lattice of " +
                    std::to_string(ctx->k.N) + " nodes");
  double* stage = nullptr;
  int rc = stageAddress(ctx, &stage);
  if (rc) return rc;
  // Waits for the work enqueued so far without reading the run's device
  // error bits: the nodes can still be read after a step reported a fault
  // (non-finite values, list overflow), which is when a monitor wants them.
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return fail(ctx, LBDEM_ERR_CUDA,
                std::string("lbdem_download_nodes_noalloc: ") + cudaGetErrorString(e));
  if (count == 0 || (!f && !mass)) return LBDEM_OK;
  const int n = (int)count;
  const int block = 256;
  const int grid = (n + block - 1) / block;
  exportNodeRange<<<grid, block, 0, ctx->stream>>>(ctx->k, ctx->d.mask, ctx->d.f[ctx->cur],
                                                   ctx->d.mass, ctx->d.nF, first, n, stage);
  e = cudaGetLastError();
  if (e == cudaSuccess && f)
    e = cudaMemcpyAsync(f, stage, (size_t)Q * n * sizeof(double), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess && mass)
    e = cudaMemcpyAsync(mass, stage + (size_t)Q * n, (size_t)n * sizeof(double),
                        cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return fail(ctx, LBDEM_ERR_CUDA,
                std::string("lbdem_download_nodes_noalloc: ") + cudaGetErrorString(e));
  ctx->launches += 1;
  return LBDEM_OK;
}
