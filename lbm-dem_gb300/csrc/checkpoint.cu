// lbdem_checkpoint / lbdem_restore: a full-precision snapshot of one run.
//
// The reference resumes a run from text files of its own: the fluid recycle
// file (IO::exportRecycleFluid, src/IO.cpp:973-997, read back by
// LB::restartInterface / LB::restartVariables, src/LB.cpp:994-1138) and the
// particle file (IO::exportRecycleParticles, src/IO.cpp:999). Those files
// keep six significant digits and drop the neighbour lists, the tangential
// springs and the step counters, so a resumed run follows a different
// trajectory. The snapshot here keeps every bit: a resumed run continues
// exactly as the uninterrupted one (up to the order of floating-point
// atomic sums, which no two runs share).
//
// File layout (host byte order):
//   Header (fixed size, below)
//   uint64 size of each device buffer, in the run's allocation order
//   the bytes of each device buffer, in the same order
// The run's device buffers are listed in lbdem_ctx::buffers as they are
// allocated; two runs created from one configuration in one form allocate
// the same buffers in the same order, which is what lets a snapshot of one
// be loaded into the other. Every size is checked before anything is
// overwritten.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "kernels_decl.h"
#include "lbdem_internal.h"

using namespace lbdem;

namespace {

constexpr char kMagic[8] = {'L', 'B', 'D', 'E', 'M', 'C', 'K', '1'};
constexpr uint32_t kVersion = 1;
constexpr uint32_t kByteOrder = 0x01020304u;
constexpr size_t kStageBytes = size_t(32) << 20;  // pinned staging per copy

struct Header {
  char magic[8];
  uint32_t version, byteOrder;
  uint32_t constsBytes;  // sizeof(Consts) of the writing library
  int32_t precision;
  int32_t X, Y, Z;
  int32_t nPart, nObj, nWall;
  int32_t flags;  // bit 0 demSolve, 1 lbSolve, 2 freeSurface
  uint64_t nBuffers, payloadBytes;
  // host-side step state
  int32_t cur, lbFReset;
  int64_t lbTime, demTimeStep;
  double demTime;
};

int fail(lbdem_ctx* ctx, int code, const std::string& msg) {
  ctx->err = msg;
  return code;
}

int runFlags(const lbdem_ctx* c) {
  return (c->demSolve ? 1 : 0) | (c->lbSolve ? 2 : 0) | (c->freeSurface ? 4 : 0);
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

struct Pinned {
  void* p = nullptr;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

#define CKC(call)                                                                 \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess)                                                        \
      return fail(ctx, LBDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

}  // namespace

extern "C" int lbdem_checkpoint(lbdem_ctx* ctx, const char* path) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  if (!path) return fail(ctx, LBDEM_ERR_INVALID, "checkpoint: null path");
  // everything enqueued so far is part of the state
  CKC(cudaStreamSynchronize(ctx->stream));
  Header h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kMagic, sizeof(kMagic));
  h.version = kVersion;
  h.byteOrder = kByteOrder;
  h.constsBytes = (uint32_t)sizeof(Consts);
  h.precision = ctx->precision;
  h.X = ctx->k.X;
  h.Y = ctx->k.Y;
  h.Z = ctx->k.Z;
  h.nPart = ctx->nPart;
  h.nObj = ctx->nObj;
  h.nWall = ctx->nWall;
  h.flags = runFlags(ctx);
  h.nBuffers = ctx->buffers.size();
  for (const auto& b : ctx->buffers) h.payloadBytes += b.second;
  h.cur = ctx->cur;
  h.lbFReset = ctx->lbFReset ? 1 : 0;
  h.lbTime = ctx->lbTime;
  h.demTimeStep = ctx->demTimeStep;
  h.demTime = ctx->demTime;

  File out;
  out.f = fopen(path, "wb");
  if (!out.f) return fail(ctx, LBDEM_ERR_IO, std::string("checkpoint: cannot open ") + path);
  bool ok = fwrite(&h, sizeof(h), 1, out.f) == 1;
  ok = ok && fwrite(&ctx->k, sizeof(Consts), 1, out.f) == 1;
  for (const auto& b : ctx->buffers) {
    const uint64_t sz = b.second;
    ok = ok && fwrite(&sz, sizeof(sz), 1, out.f) == 1;
  }
  if (!ok) return fail(ctx, LBDEM_ERR_IO, std::string("checkpoint: write failed: ") + path);
  Pinned stage;
  CKC(cudaMallocHost(&stage.p, kStageBytes));
  for (const auto& b : ctx->buffers) {
    for (size_t off = 0; off < b.second; off += kStageBytes) {
      const size_t n = std::min(kStageBytes, b.second - off);
      CKC(cudaMemcpyAsync(stage.p, (const char*)b.first + off, n, cudaMemcpyDeviceToHost,
                          ctx->stream));
      CKC(cudaStreamSynchronize(ctx->stream));
      if (fwrite(stage.p, 1, n, out.f) != n)
        return fail(ctx, LBDEM_ERR_IO, std::string("checkpoint: write failed: ") + path);
    }
  }
  if (fflush(out.f) != 0)
    return fail(ctx, LBDEM_ERR_IO, std::string("checkpoint: write failed: ") + path);
  return LBDEM_OK;
}

extern "C" int lbdem_restore(lbdem_ctx* ctx, const char* path) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  if (!path) return fail(ctx, LBDEM_ERR_INVALID, "restore: null path");
  File in;
  in.f = fopen(path, "rb");
  if (!in.f) return fail(ctx, LBDEM_ERR_IO, std::string("restore: cannot open ") + path);
  Header h;
  if (fread(&h, sizeof(h), 1, in.f) != 1)
    return fail(ctx, LBDEM_ERR_IO, "restore: file shorter than the snapshot header");
  if (std::memcmp(h.magic, kMagic, sizeof(kMagic)) != 0)
    return fail(ctx, LBDEM_ERR_IO, "restore: not a snapshot file");
  if (h.version != kVersion || h.byteOrder != kByteOrder || h.constsBytes != sizeof(Consts))
    return fail(ctx, LBDEM_ERR_INVALID,
                "restore: snapshot written by an incompatible library build or byte order");
  auto mismatch = [&](const char* what, long long a, long long b) {
    return fail(ctx, LBDEM_ERR_INVALID,
                std::string("restore: snapshot ") + what + " " + std::to_string(a) +
                    " differs from this run's " + std::to_string(b));
  };
  if (h.precision != ctx->precision) return mismatch("precision", h.precision, ctx->precision);
  if (h.X != ctx->k.X) return mismatch("lattice X", h.X, ctx->k.X);
  if (h.Y != ctx->k.Y) return mismatch("lattice Y", h.Y, ctx->k.Y);
  if (h.Z != ctx->k.Z) return mismatch("lattice Z", h.Z, ctx->k.Z);
  if (h.nPart != ctx->nPart) return mismatch("particle count", h.nPart, ctx->nPart);
  if (h.nObj != ctx->nObj) return mismatch("object count", h.nObj, ctx->nObj);
  if (h.nWall != ctx->nWall) return mismatch("wall count", h.nWall, ctx->nWall);
  if (h.flags != runFlags(ctx)) return mismatch("solver switches", h.flags, runFlags(ctx));
  if (h.nBuffers != ctx->buffers.size())
    return mismatch("buffer count", (long long)h.nBuffers, (long long)ctx->buffers.size());
  Consts k;
  if (fread(&k, sizeof(Consts), 1, in.f) != 1)
    return fail(ctx, LBDEM_ERR_IO, "restore: file truncated in the run constants");
  for (size_t i = 0; i < ctx->buffers.size(); ++i) {
    uint64_t sz = 0;
    if (fread(&sz, sizeof(sz), 1, in.f) != 1)
      return fail(ctx, LBDEM_ERR_IO, "restore: file truncated in the buffer table");
    if (sz != ctx->buffers[i].second)
      return mismatch(("buffer " + std::to_string(i) + " size").c_str(), (long long)sz,
                      (long long)ctx->buffers[i].second);
  }
  // the payload must be complete before any device buffer is overwritten
  const long dataStart = ftell(in.f);
  if (dataStart < 0 || fseek(in.f, 0, SEEK_END) != 0)
    return fail(ctx, LBDEM_ERR_IO, "restore: cannot seek in the snapshot");
  const long end = ftell(in.f);
  if (end < 0 || (uint64_t)(end - dataStart) != h.payloadBytes)
    return fail(ctx, LBDEM_ERR_IO, "restore: snapshot payload has the wrong length");
  if (fseek(in.f, dataStart, SEEK_SET) != 0)
    return fail(ctx, LBDEM_ERR_IO, "restore: cannot seek in the snapshot");

  CKC(cudaStreamSynchronize(ctx->stream));
  if (int rc = lbdemOutputDrain(ctx, true)) return rc;  // lines of the run being replaced
  Pinned stage;
  CKC(cudaMallocHost(&stage.p, kStageBytes));
  for (const auto& b : ctx->buffers) {
    for (size_t off = 0; off < b.second; off += kStageBytes) {
      const size_t n = std::min(kStageBytes, b.second - off);
      if (fread(stage.p, 1, n, in.f) != n)
        return fail(ctx, LBDEM_ERR_IO, "restore: read failed in the payload");
      CKC(cudaMemcpyAsync((char*)b.first + off, stage.p, n, cudaMemcpyHostToDevice,
                          ctx->stream));
      CKC(cudaStreamSynchronize(ctx->stream));
    }
  }
  // run constants as they were (the lbF reset of the first collision), with
  // this run's own device pointers
  k.chunkAct = ctx->k.chunkAct;
  ctx->k = k;
  ctx->cur = h.cur;
  ctx->lbFReset = h.lbFReset != 0;
  ctx->lbTime = h.lbTime;
  ctx->demTimeStep = h.demTimeStep;
  ctx->demTime = h.demTime;
  // open output files continue from the restored cycle count
  lbdemOutputResync(ctx);
  // captured cycles hold the old constants by value: capture again
  for (auto& g : ctx->pairGraph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& g : ctx->oneGraph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& row : ctx->groupGraph)
    for (auto& g : row)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  return LBDEM_OK;
}
