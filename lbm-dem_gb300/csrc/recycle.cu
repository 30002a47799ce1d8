// The reference's fluid recycle file: writer (IO::exportRecycleFluid,
// src/IO.cpp:973-997) and reader (LB::restartInterface and
// LB::restartVariables under lbRestart, src/LB.cpp:353-367, 994-1138).
//
// Format (text, the stream's default six significant digits):
//   "X Y Z\n"
//   the type of every node in index order, each followed by a space, "\n"
//   per active node (fluid or interface) in index order:
//     n - rho0, ux, uy, uz, mass - rho0, visc, f_0 .. f_18, each followed by
//     a space, then "\n"
// The writer's node order is LB::activeNodes after LB::cleanLists, which
// sorts it (src/LB.cpp:1226-1231); cleanLists closes every free-surface
// step, so at a cycle's end it is the fluid and interface nodes by index.
// Its n and u columns are the reference's node fields, the density and the
// force-shifted velocity of the last collision; this writer gives the
// density and velocity of the current populations instead (the collision's
// values of particle nodes depend on a mass the run no longer holds). A
// restart reads neither column.
//
// Reading, as the reference does after LB::initializeTypes: every node that
// the geometry leaves fluid takes the file's type (walls, impactors keep
// theirs); then, for every node active under those types, in index order,
// the next record gives its populations and its mass (node::restart,
// src/node.cpp:38-50). n and u of the record are not used: the lattice step
// recomputes them from the populations before any use. Its viscosity is
// the node's in a run with a per-node viscosity (non-Newtonian rheology or
// turbulence); a Newtonian run has one viscosity, the configuration's.
#include <cuda_runtime.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lattice_common.cuh"

using namespace lbdem;

namespace {

int fail(lbdem_ctx* ctx, int code, const std::string& msg) {
  ctx->err = msg;
  return code;
}

// whitespace-separated numbers of a whole file
struct Tokens {
  std::vector<char> buf;
  const char* p = nullptr;
  const char* end = nullptr;
  bool load(const char* path) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(n > 0 ? (size_t)n + 1 : 1);
    const size_t got = n > 0 ? std::fread(buf.data(), 1, (size_t)n, f) : 0;
    std::fclose(f);
    buf[got] = '\0';
    p = buf.data();
    end = buf.data() + got;
    return true;
  }
  bool num(double& v) {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r')) ++p;
    if (p >= end) return false;
    char* e = nullptr;
    v = std::strtod(p, &e);
    if (e == p) return false;
    p = e;
    return true;
  }
  bool uint(unsigned& v) {
    double d;
    if (!num(d) || d < 0.0 || d != (double)(unsigned)d) return false;
    v = (unsigned)d;
    return true;
  }
};

}  // namespace

// Called by lbdem_create under lbRestart, after initTypes has typed the
// lattice as LB::initializeTypes does (no free-surface interface).
int lbdemRestartFluid(lbdem_ctx* ctx, const char* path) {
  if (!path || !*path) return fail(ctx, LBDEM_ERR_INVALID, "lbRestart without lbRestartFile");
  Tokens in;
  if (!in.load(path)) return fail(ctx, LBDEM_ERR_IO, std::string("cannot open ") + path);
  const Consts& k = ctx->k;
  const size_t N = (size_t)k.N, NP = (size_t)k.NP;
  unsigned X = 0, Y = 0, Z = 0;
  if (!in.uint(X) || !in.uint(Y) || !in.uint(Z))
    return fail(ctx, LBDEM_ERR_IO, std::string("restart file: no lattice size in ") + path);
  if ((int)X != k.X || (int)Y != k.Y || (int)Z != k.Z)  // src/LB.cpp:363-365
    return fail(ctx, LBDEM_ERR_INVALID, "restart file: lattice size differs from the run's");
  cudaStream_t st = ctx->stream;
  Device& d = ctx->d;
  std::vector<uint8_t> mask(N);
  cudaError_t e = cudaMemcpyAsync(mask.data(), d.mask, N, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(ctx, LBDEM_ERR_CUDA, cudaGetErrorString(e));
  // LB::restartInterface: fluid nodes take the file's type
  for (size_t x = 0; x < N; ++x) {
    unsigned t = 0;
    if (!in.uint(t) || t > TYPE_MASK)
      return fail(ctx, LBDEM_ERR_IO, "restart file: bad or missing node type");
    // a node the file makes an impactor node lies outside the impactor
    // (the geometry left it fluid): the reference never adds it to its
    // object node list
    if ((mask[x] & TYPE_MASK) == 0)
      mask[x] = (uint8_t)((mask[x] & ~TYPE_MASK) | t | (t == 12 ? OSTALE : 0));
  }
  // LB::restartVariables, then the active-list bit of the first cleanLists
  const double rho0 = k.initDensity;
  std::vector<double> mass(N, 0.0);
  std::vector<double> visc;
  if (d.visc) visc.assign(N, k.initVisc);
  std::vector<double> f64;
  std::vector<float> f32, nF;
  if (k.mixed) {
    f32.assign((size_t)Q * NP, 0.0f);
    nF.assign(NP, 0.0f);
  } else {
    f64.assign((size_t)Q * NP, 0.0);
  }
  for (size_t x = 0; x < N; ++x) {
    const int t = mask[x] & TYPE_MASK;
    if (t != 0 && t != 3) continue;
    double rec[6 + Q];
    for (int c = 0; c < 6 + Q; ++c)
      if (!in.num(rec[c]))
        return fail(ctx, LBDEM_ERR_IO, "restart file: fewer node records than active nodes");
    const double m = rec[4] + rho0;
    mass[x] = m;
    if (d.visc) visc[x] = rec[5];
    for (int j = 0; j < Q; ++j) {
      if (k.mixed) f32[(size_t)j * NP + x] = (float)(rec[6 + j] - WJ(j));
      else f64[(size_t)j * NP + x] = rec[6 + j];
    }
    if (k.mixed && t == 0) nF[x] = (float)m;
    mask[x] |= ABIT;
  }
  e = cudaMemcpyAsync(d.mask, mask.data(), N, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d.mass, mass.data(), N * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && d.visc)
    e = cudaMemcpyAsync(d.visc, visc.data(), N * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    if (k.mixed) {
      e = cudaMemcpyAsync(d.f[0], f32.data(), f32.size() * sizeof(float),
                          cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d.nF, nF.data(), nF.size() * sizeof(float),
                            cudaMemcpyHostToDevice, st);
    } else {
      e = cudaMemcpyAsync(d.f[0], f64.data(), f64.size() * sizeof(double),
                          cudaMemcpyHostToDevice, st);
    }
  }
  // the host arrays are freed on return
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(ctx, LBDEM_ERR_CUDA, cudaGetErrorString(e));
  return LBDEM_OK;
}

extern "C" int lbdem_export_recycle_fluid(lbdem_ctx* ctx, const char* path) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  if (!path) return fail(ctx, LBDEM_ERR_INVALID, "export_recycle_fluid: null path");
  const Consts& k = ctx->k;
  const size_t N = (size_t)k.N;
  std::vector<uint8_t> type(N);
  std::vector<double> n(N), u(3 * N), mass(N), f((size_t)Q * N);
  int rc = lbdem_download_lattice(ctx, type.data(), nullptr, nullptr, n.data(), u.data(),
                                  mass.data(), f.data());
  if (rc) return rc;
  std::vector<double> viscN;
  if (ctx->d.visc) {
    viscN.resize(N);
    if ((rc = lbdem_download_viscosity(ctx, viscN.data()))) return rc;
  }
  std::FILE* out = std::fopen(path, "w");
  if (!out) return fail(ctx, LBDEM_ERR_IO, std::string("cannot write ") + path);
  const double rho0 = k.initDensity, visc = k.initVisc;
  std::fprintf(out, "%d %d %d\n", k.X, k.Y, k.Z);
  for (size_t x = 0; x < N; ++x) std::fprintf(out, "%d ", (int)type[x]);
  std::fputs("\n", out);
  for (size_t x = 0; x < N; ++x) {
    if (type[x] != 0 && type[x] != 3) continue;
    std::fprintf(out, "%g %g %g %g %g %g ", n[x] - rho0, u[x], u[N + x], u[2 * N + x],
                 mass[x] - rho0, viscN.empty() ? visc : viscN[x]);
    for (int j = 0; j < Q; ++j) std::fprintf(out, "%g ", f[(size_t)j * N + x]);
    std::fputs("\n", out);
  }
  const bool ok = std::ferror(out) == 0;
  if (std::fclose(out) != 0 || !ok)
    return fail(ctx, LBDEM_ERR_IO, std::string("write failed: ") + path);
  return LBDEM_OK;
}
