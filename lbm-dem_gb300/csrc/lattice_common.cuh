// Lattice helpers shared by the FP64 and the mixed-precision kernels:
// the D3Q19 set in the reference's order, index arithmetic, the exact FP64
// node collision, the FP32-deviation node collision, population storage
// accessors and the warp-level particle reduction.
#pragma once
#include <cfloat>
#include <climits>

#include "kernels_decl.h"

namespace lbdem {

// D3Q19 velocity set in the reference's order, src/lattice.h:33-57
__host__ __device__ constexpr int CX(int j) {
  return j == 1 ? 1 : j == 2 ? -1 : j == 7 ? 1 : j == 8 ? -1 : j == 9 ? -1 : j == 10 ? 1
       : j == 15 ? 1 : j == 16 ? -1 : j == 17 ? 1 : j == 18 ? -1 : 0;
}
__host__ __device__ constexpr int CY(int j) {
  return j == 3 ? 1 : j == 4 ? -1 : j == 7 ? 1 : j == 8 ? -1 : j == 9 ? 1 : j == 10 ? -1
       : j == 11 ? 1 : j == 12 ? -1 : j == 13 ? -1 : j == 14 ? 1 : 0;
}
__host__ __device__ constexpr int CZ(int j) {
  return j == 5 ? 1 : j == 6 ? -1 : j == 11 ? 1 : j == 12 ? -1 : j == 13 ? 1 : j == 14 ? -1
       : j == 15 ? 1 : j == 16 ? -1 : j == 17 ? -1 : j == 18 ? 1 : 0;
}
__host__ __device__ constexpr int OPPJ(int j) { return j == 0 ? 0 : (j & 1) ? j + 1 : j - 1; }
// weights, src/lattice.h:147-150 (same double values as 12/36, 2/36, 1/36)
__host__ __device__ constexpr double WJ(int j) {
  return j == 0 ? 12.0 / 36.0 : j <= 6 ? 2.0 / 36.0 : 1.0 / 36.0;
}

__host__ __device__ __forceinline__ bool isActiveT(int t) { return t == 0 || t == 3; }

// bits j = 1..18 of the links whose lattice velocity has the given component sign
__host__ __device__ constexpr unsigned linksWith(int axis, int sign) {
  unsigned m = 0;
  for (int j = 1; j < 19; ++j) {
    const int c = axis == 0 ? CX(j) : axis == 1 ? CY(j) : CZ(j);
    if (c == sign) m |= 1u << j;
  }
  return m;
}

// A node became active outside the lattice step (free-surface filling, an
// uncovered impactor node): flag its warp of its 256-node chunk so that the
// next mixed lattice step does not skip the chunk.
__device__ __forceinline__ void markActive(const Consts& k, long long x) {
  if (k.chunkAct) atomicOr(k.chunkAct + (x >> 8), 1u << ((x >> 5) & 7));
}

// Links of node (ix, iy, iz) that end in the outer node layer of the box.
// A run accepts walls on all six faces and no other boundary, so the outer
// layer is all wall nodes and these are exactly the node's wall links.
__device__ __forceinline__ unsigned boxWallLinks(const Consts& k, int ix, int iy, int iz) {
  unsigned w = 0;
  if (ix == 1) w |= linksWith(0, -1);
  if (ix == k.X - 2) w |= linksWith(0, 1);
  if (iy == 1) w |= linksWith(1, -1);
  if (iy == k.Y - 2) w |= linksWith(1, 1);
  if (iz == 1) w |= linksWith(2, -1);
  if (iz == k.Z - 2) w |= linksWith(2, 1);
  return w;
}

// u.dot(v[j]) of src/myvector.cpp:121 with the zero components dropped
__device__ __forceinline__ double dotc(int j, double x, double y, double z) {
  const int cx = CX(j), cy = CY(j), cz = CZ(j);
  double s = 0.0;
  bool any = false;
  if (cx) { s = cx > 0 ? x : -x; any = true; }
  if (cy) { const double t = cy > 0 ? y : -y; s = any ? s + t : t; any = true; }
  if (cz) { const double t = cz > 0 ? z : -z; s = any ? s + t : t; }
  return s;
}

__device__ __forceinline__ long long nbrOffset(const Consts& k, int j) {
  return (long long)CX(j) + (long long)CY(j) * k.sy + (long long)CZ(j) * k.sz;
}

// Appends node x to the interface list. Called only by the lanes that hold
// an interface node; the lanes executing together share one atomic and
// write their entries in lane order.
__device__ __forceinline__ void appendInterface(uint32_t x, uint32_t* list, int* iscal) {
  const unsigned am = __activemask();
  const int lane = threadIdx.x & 31, first = __ffs(am) - 1;
  int base = 0;
  if (lane == first) base = atomicAdd(iscal + IS_IFLIST, __popc(am));
  base = __shfl_sync(am, base, first);
  list[base + __popc(am & ((1u << lane) - 1u))] = x;
}

__device__ __forceinline__ void coords(const Consts& k, long long x, int& ix, int& iy, int& iz) {
  const unsigned ux = (unsigned)x;
  iz = (int)(ux / (unsigned)k.sz);
  const unsigned rem = ux - (unsigned)iz * (unsigned)k.sz;
  iy = (int)(rem / (unsigned)k.X);
  ix = (int)(rem - (unsigned)iy * (unsigned)k.X);
}

// Compensated accumulation of a mass-budget sum: the atomic addition's
// rounding error, formed from the value it replaced (TwoSum; exact without
// contraction), goes to a second accumulator; the budget is acc + lo.
__device__ __forceinline__ void atomicAddComp(double* acc, double* lo, double v) {
  const double old = atomicAdd(acc, v);
  const double s = __dadd_rn(old, v);
  const double bp = __dsub_rn(s, old);
  const double err = __dadd_rn(__dsub_rn(old, __dsub_rn(s, bp)), __dsub_rn(v, bp));
  if (err != 0.0) atomicAdd(lo, err);
}

// tinyVector::insideSphere, src/myvector.cpp:171-176, on node coordinates
__device__ __forceinline__ bool insideSphere(double px, double py, double pz, double cx,
                                             double cy, double cz, double r) {
  const double dx = px - cx, dy = py - cy, dz = pz - cz;
  return dx * dx + dy * dy + dz * dz < r * r;
}
// insideSphere for the nodes of a box: the centre is kept relative to the
// box corner lo, where an FP32 squared distance is within about 1e-5 (lu^2)
// of the FP64 one for spheres of a few lattice units. Outside a band of
// r^2 * 1e-5 + 3e-5 around r^2 the FP32 comparison gives the FP64 answer;
// inside it the FP64 test decides.
struct SphereBoxTest {
  double cx, cy, cz, r;
  int lo[3];
  float fx, fy, fz, r2in, r2out;
};
__device__ __forceinline__ SphereBoxTest sphereBoxTest(double cx, double cy, double cz,
                                                       double r, const int* lo) {
  SphereBoxTest t;
  t.cx = cx;
  t.cy = cy;
  t.cz = cz;
  t.r = r;
  for (int a = 0; a < 3; ++a) t.lo[a] = lo[a];
  t.fx = (float)(cx - (double)lo[0]);
  t.fy = (float)(cy - (double)lo[1]);
  t.fz = (float)(cz - (double)lo[2]);
  const float r2 = (float)r * (float)r;
  const float band = r2 * 1e-5f + 3e-5f;
  t.r2in = r2 - band;
  t.r2out = r2 + band;
  return t;
}
__device__ __forceinline__ bool insideBox(const SphereBoxTest& t, int ix, int iy, int iz) {
  const float dx = (float)(ix - t.lo[0]) - t.fx;
  const float dy = (float)(iy - t.lo[1]) - t.fy;
  const float dz = (float)(iz - t.lo[2]) - t.fz;
  const float d2 = dx * dx + dy * dy + dz * dz;
  if (d2 < t.r2in) return true;
  if (d2 > t.r2out) return false;
  return insideSphere((double)ix, (double)iy, (double)iz, t.cx, t.cy, t.cz, t.r);
}
// The same answer with FP32 arithmetic where it is clear: the FP32 squared
// distance is within a few 1e-7 (relative) of the FP64 one, so outside a
// relative band of 4e-6 around r^2 the comparison cannot differ; inside the
// band the FP64 test decides.
__device__ __forceinline__ bool insideSphereFast(double px, double py, double pz, double cx,
                                                 double cy, double cz, double r) {
  const float dx = (float)(px - cx), dy = (float)(py - cy), dz = (float)(pz - cz);
  const float d2 = dx * dx + dy * dy + dz * dz;
  const float r2 = (float)r * (float)r;
  if (d2 < r2 * (1.0f - 4e-6f)) return true;
  if (d2 > r2 * (1.0f + 4e-6f)) return false;
  return insideSphere(px, py, pz, cx, cy, cz, r);
}

// node::setEquilibrium / computeEquilibrium for one direction,
// src/node.cpp:52-73, 100-111
__device__ __forceinline__ double feqj(int j, double n, double ux, double uy, double uz,
                                       double usq) {
  const double vu = dotc(j, ux, uy, uz);
  return WJ(j) * n * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
}

// One node's collision, exactly as LB::reconstruction + computeHydroForces
// (node part) + LB::collision: in f = pre-collision populations, out f =
// post-collision populations (fs). Returns n, the shifted u, the node force.
struct NodeState {
  double n, ux, uy, uz, hx, hy, hz;
  // particle coupling terms for the per-particle reduction
  double dx, dy, dz, rx, ry, rz;
};

// node::computeApparentViscosity (src/node.cpp:113-168) on the node's
// pre-collision populations f, its equilibrium feq, density n and shifted
// velocity; visc is the node's viscosity of the last step (tau) and gets the
// new one. Same operations and order as the reference (this is compiled
// without FMA contraction); terms with c_a c_b = 0 are skipped (they add an
// exact +-0), c_a c_b = -1 subtracts.
__device__ __forceinline__ void apparentViscosity(const Consts& k, const double* f,
                                                  const double* feq, double n, double ux,
                                                  double uy, double uz, double& visc) {
  const double minVisc = (0.500001 - 0.5) / 3.0;  // minTau, src/lattice.h:26
  const double maxVisc = (1.8 - 0.5) / 3.0;       // maxTau, src/lattice.h:27
  const double tau = 0.5 + 3.0 * visc;
  double g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int j = 0; j < Q; ++j) {
    const double d = f[j] - feq[j];
    const int c[3] = {CX(j), CY(j), CZ(j)};
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int cc = c[p] * c[q];
        if (cc > 0) g[3 * p + q] += d;
        else if (cc < 0) g[3 * p + q] += -d;
      }
  }
  const double sc = 1.5 / (tau * n);
#pragma unroll
  for (int i = 0; i < 9; ++i) g[i] *= sc;
  // tinyMatrix::magnitude, src/myvector.cpp:546-550
  const double mag = sqrt(0.5 * (g[0] * g[0] + g[4] * g[4] + g[8] * g[8] +
                                 2.0 * (g[1] * g[3] + g[6] * g[2] + g[5] * g[7])));
  const double shearRate = 2.0 * mag;
  double nuApp;
  if (k.rheo == LBDEM_BINGHAM) {
    nuApp = k.plasticVisc + k.yieldStress / shearRate;
  } else if (k.rheo == LBDEM_FRICTIONAL) {
    const double pr = 0.33333333 * (n - 1.0);
    const double pressure = pr > 0.0 ? pr : 0.0;  // std::max(0.0, pr)
    nuApp = k.initVisc + k.frictionCoef * pressure / shearRate;
  } else if (k.rheo == LBDEM_VOELLMY) {
    const double pr = 0.33333333 * (n - 1.0);
    const double pressure = pr > 0.0 ? pr : 0.0;
    nuApp = (k.frictionCoef * pressure + (ux * ux + uy * uy + uz * uz) / k.voellmyCoef) /
            shearRate;
  } else {
    nuApp = k.initVisc;
  }
  if (k.turbulence) {
    const double nuTurb = k.turbConst * shearRate;
    nuApp += nuTurb;
  }
  // std::max(minVisc, std::min(maxVisc, nuApp)), NaN handling included
  const double lo = nuApp < maxVisc ? nuApp : maxVisc;
  visc = minVisc < lo ? lo : minVisc;
}

// RHEO: the node's viscosity comes from viscp (k.visc + x) instead of the
// run's single value; with update, the apparent viscosity is evaluated
// first and stored there (LB::collision, src/LB.cpp:1322-1325), otherwise
// the stored one is used (a recomputation of the same collision).
template <bool RHEO = false>
__device__ __forceinline__ void collideNode(const Consts& k, double* f, bool pflag,
                                            uint32_t pid, const double* px0,
                                            const double* px1, const double* pw1,
                                            int P, double massOld, int ix, int iy, int iz,
                                            NodeState& s, double* viscp = nullptr,
                                            bool update = false) {
  // node::reconstruct
  double n = 0.0;
#pragma unroll
  for (int j = 0; j < Q; ++j) n += f[j];
  double ux = 0.0, uy = 0.0, uz = 0.0;
  {
    bool ax = false, ay = false, az = false;
#pragma unroll
    for (int j = 1; j < Q; ++j) {
      if (CX(j)) { const double t = CX(j) > 0 ? f[j] : -f[j]; ux = ax ? ux + t : t; ax = true; }
      if (CY(j)) { const double t = CY(j) > 0 ? f[j] : -f[j]; uy = ay ? uy + t : t; ay = true; }
      if (CZ(j)) { const double t = CZ(j) > 0 ? f[j] : -f[j]; uz = az ? uz + t : t; az = true; }
    }
  }
  ux /= n;
  uy /= n;
  uz /= n;
  // LB::computeHydroForces, node part (src/LB.cpp:1920-1940)
  double hx = 0.0, hy = 0.0, hz = 0.0;
  s.dx = s.dy = s.dz = 0.0;
  s.rx = s.ry = s.rz = 0.0;
  if (pflag && pid < (uint32_t)P) {
    // px0 = x0/unit.Length and px1 = x1/unit.Speed, divided once per particle
    // (particleKinematics); the quotients are the same bits the reference
    // computes at every node.
    const double rx = (double)ix - px0[pid];
    const double ry = (double)iy - px0[P + pid];
    const double rz = (double)iz - px0[2 * P + pid];
    const double wx = pw1[pid], wy = pw1[P + pid], wz = pw1[2 * P + pid];
    const double lvx = px1[pid] + (wy * rz - wz * ry) / k.uAngVel;
    const double lvy = px1[P + pid] + (wz * rx - wx * rz) / k.uAngVel;
    const double lvz = px1[2 * P + pid] + (wx * ry - wy * rx) / k.uAngVel;
    const double lf = massOld / n;
    s.dx = (ux - lvx) * lf;
    s.dy = (uy - lvy) * lf;
    s.dz = (uz - lvz) * lf;
    s.rx = rx;
    s.ry = ry;
    s.rz = rz;
    hx = 0.0 + s.dx * -1.0;
    hy = 0.0 + s.dy * -1.0;
    hz = 0.0 + s.dz * -1.0;
  }
  // node::shiftVelocity
  const double Tx = k.lbF[0] + hx, Ty = k.lbF[1] + hy, Tz = k.lbF[2] + hz;
  ux = ux + Tx * 0.5 / n;
  uy = uy + Ty * 0.5 / n;
  uz = uz + Tz * 0.5 / n;
  const double usq = ux * ux + uy * uy + uz * uz;
  double omega = k.omega, omegaf = k.omegaf;
  if (RHEO) {
    double visc = *viscp;
    if (update) {
      double feqa[Q];
#pragma unroll
      for (int j = 0; j < Q; ++j) {
        const double vu = dotc(j, ux, uy, uz);
        feqa[j] = WJ(j) * n * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
      }
      apparentViscosity(k, f, feqa, n, ux, uy, uz, visc);
      *viscp = visc;
    }
    omega = 1.0 / (0.5 + 3.0 * visc);          // node::solveCollision
    omegaf = 1.0 - 1.0 / (1.0 + 6.0 * visc);   // node::addForce
  }
  // node::solveCollision + node::addForce
#pragma unroll
  for (int j = 0; j < Q; ++j) {
    const double vu = dotc(j, ux, uy, uz);
    const double feq = WJ(j) * n * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
    double fj = f[j] + omega * (feq - f[j]);
    const double v9 = 9.0 * vu;
    const double fpx = CX(j) == 0 ? (-ux) * 3.0 : CX(j) > 0 ? v9 + (1.0 - ux) * 3.0
                                                             : -v9 + (-1.0 - ux) * 3.0;
    const double fpy = CY(j) == 0 ? (-uy) * 3.0 : CY(j) > 0 ? v9 + (1.0 - uy) * 3.0
                                                             : -v9 + (-1.0 - uy) * 3.0;
    const double fpz = CZ(j) == 0 ? (-uz) * 3.0 : CZ(j) > 0 ? v9 + (1.0 - uz) * 3.0
                                                             : -v9 + (-1.0 - uz) * 3.0;
    fj += omegaf * WJ(j) * (fpx * Tx + fpy * Ty + fpz * Tz);
    f[j] = fj;
  }
  s.n = n;
  s.ux = ux;
  s.uy = uy;
  s.uz = uz;
  s.hx = hx;
  s.hy = hy;
  s.hz = hz;
}


// per-block accumulator layout in shared memory
enum { ACC_WALL = 0, ACC_OBJ = ACC_WALL + 3 * MAX_WALL, ACC_EXTRA = ACC_OBJ + 6 * MAX_OBJ,
       ACC_N = ACC_EXTRA + 1 };

// Reduce 16 per-lane particle terms over the lanes of a warp that share a
// particle index and add them to the particle's accumulators.
__device__ __forceinline__ void warpParticleReduce(int key, const double* v, double* pF,
                                                   double* pM, double* pS, double* pV,
                                                   int P) {
  const unsigned FULL = 0xffffffffu;
  unsigned todo = __ballot_sync(FULL, key >= 0);
  const int lane = threadIdx.x & 31;
  while (todo) {
    const int leader = __ffs(todo) - 1;
    const int kk = __shfl_sync(FULL, key, leader);
    const bool mine = key == kk;
    const unsigned grp = __ballot_sync(FULL, mine);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      double x = mine ? v[i] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
      if (lane == leader) {
        double* dst = i < 3 ? pF + i * P : i < 6 ? pM + (i - 3) * P : i < 15 ? pS + (i - 6) * P
                                                                               : pV;
        atomicAdd(dst + kk, x);
      }
    }
    todo &= ~grp;
  }
}

// Per-thread accumulation of the bounce-back force sums. The wall and the
// impactor a thread last touched are kept in registers and flushed to the
// block's shared accumulators only when the index changes and at the end,
// instead of one shared-memory atomic per boundary link.
template <typename WT>
struct BBAccT {
  int wId = -1, oId = -1;
  WT w[3] = {0, 0, 0};
  double o[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double extra = 0.0;
  __device__ __forceinline__ void flushWall(double* acc) {
    if (wId >= 0)
      for (int c = 0; c < 3; ++c)
        if (w[c] != 0) {
          atomicAdd(&acc[ACC_WALL + 3 * wId + c], (double)w[c]);
          w[c] = 0;
        }
  }
  __device__ __forceinline__ void flushObj(double* acc) {
    if (oId >= 0)
      for (int c = 0; c < 6; ++c)
        if (o[c] != 0.0) {
          atomicAdd(&acc[ACC_OBJ + 6 * oId + c], o[c]);
          o[c] = 0.0;
        }
  }
  __device__ __forceinline__ void wall(double* acc, int id, int c, WT v) {
    if (id != wId) {
      flushWall(acc);
      wId = id;
    }
    w[c] += v;
  }
  __device__ __forceinline__ void obj(double* acc, int id, int c, double v) {
    if (id != oId) {
      flushObj(acc);
      oId = id;
    }
    o[c] += v;
  }
  __device__ __forceinline__ void flush(double* acc) {
    flushWall(acc);
    flushObj(acc);
    if (extra != 0.0) atomicAdd(&acc[ACC_EXTRA], extra);
    extra = 0.0;
  }
};
using BBAcc = BBAccT<double>;   // plain form
using BBAccF = BBAccT<float>;   // mixed form: wall sums (diagnostic) in float

// ---- population storage ------------------------------------------------------
// Plain form: f itself in double. Mixed form: the deviation f - w_j in float
// (w_j = initDensity * weight, initDensity is 1 in the reference,
// src/LB.cpp:330), which keeps the float's precision for the part that
// varies.
__device__ __forceinline__ double fget(const Consts& k, const void* f, int j, long long x) {
  return k.mixed ? (double)((const float*)f)[(long long)j * k.NP + x] + WJ(j)
                 : ((const double*)f)[(long long)j * k.NP + x];
}
__device__ __forceinline__ void fset(const Consts& k, void* f, int j, long long x, double v) {
  if (k.mixed) ((float*)f)[(long long)j * k.NP + x] = (float)(v - WJ(j));
  else ((double*)f)[(long long)j * k.NP + x] = v;
}
// f_j1(x1) - f_j2(x2) for two directions of equal weight
__device__ __forceinline__ double fdiff(const Consts& k, const void* f, int j1, long long x1,
                                        int j2, long long x2) {
  if (k.mixed)
    return (double)((const float*)f)[(long long)j1 * k.NP + x1] -
           (double)((const float*)f)[(long long)j2 * k.NP + x2];
  return ((const double*)f)[(long long)j1 * k.NP + x1] -
         ((const double*)f)[(long long)j2 * k.NP + x2];
}

// u.dot(v[j]) in float
__device__ __forceinline__ float dotcf(int j, float x, float y, float z) {
  float s = 0.0f;
  if (CX(j)) s = CX(j) > 0 ? x : -x;
  if (CY(j)) s = CY(j) > 0 ? s + y : s - y;
  if (CZ(j)) s = CZ(j) > 0 ? s + z : s - z;
  return s;
}

struct NodeStateF {
  float n, ux, uy, uz, hx, hy, hz;
  float dx, dy, dz, rx, ry, rz;
};

// Float kinematics of particle pid (lbPrepare): centre x0/L, velocity x1/S
// and angular velocity w1/W, three float4 per particle.
struct KinF {
  float4 x0, x1, w1;
};
__device__ __forceinline__ KinF loadKinF(const float* pkf, uint32_t pid) {
  const float4* q = reinterpret_cast<const float4*>(pkf) + 3 * (size_t)pid;
  return KinF{__ldg(q), __ldg(q + 1), __ldg(q + 2)};
}

// Mixed form of collideNode: BGK + Guo forcing with the particle coupling of
// LB::computeHydroForces, on float deviations g = f - w (in/out). The
// particle's kinematics kin and the node's old mass are loaded by the caller
// (ahead of the moment sums, so that their latency overlaps them) and used
// when coupled is set. Explicit fused multiply-adds, so the result is the
// same in every translation unit whatever its contraction flags.
__device__ __forceinline__ void collideNodeMixed(const Consts& k, float* g, bool coupled,
                                                 const KinF& kin, float massOld, int ix,
                                                 int iy, int iz, NodeStateF& s) {
  // moments from the sums and differences of opposite pairs (j odd, j + 1)
  float dr = g[0];
  float jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
  for (int j = 1; j < Q; j += 2) {
    dr += g[j] + g[j + 1];
    const float dj = g[j] - g[j + 1];
    if (CX(j)) jx = CX(j) > 0 ? jx + dj : jx - dj;
    if (CY(j)) jy = CY(j) > 0 ? jy + dj : jy - dj;
    if (CZ(j)) jz = CZ(j) > 0 ? jz + dj : jz - dj;
  }
  const float n = 1.0f + dr;
  const float inv = __frcp_rn(n);
  float ux = jx * inv, uy = jy * inv, uz = jz * inv;
  float hx = 0.0f, hy = 0.0f, hz = 0.0f;
  s.dx = s.dy = s.dz = s.rx = s.ry = s.rz = 0.0f;
  if (coupled) {
    const float4 X0 = kin.x0, X1 = kin.x1, W1 = kin.w1;
    const float rx = (float)ix - X0.x;
    const float ry = (float)iy - X0.y;
    const float rz = (float)iz - X0.z;
    const float wx = W1.x, wy = W1.y, wz = W1.z;
    const float lvx = X1.x + __fmaf_rn(wy, rz, -wz * ry);
    const float lvy = X1.y + __fmaf_rn(wz, rx, -wx * rz);
    const float lvz = X1.z + __fmaf_rn(wx, ry, -wy * rx);
    const float lf = massOld * inv;
    s.dx = (ux - lvx) * lf;
    s.dy = (uy - lvy) * lf;
    s.dz = (uz - lvz) * lf;
    s.rx = rx;
    s.ry = ry;
    s.rz = rz;
    hx = -s.dx;
    hy = -s.dy;
    hz = -s.dz;
  }
  const float Tx = k.lbFf[0] + hx, Ty = k.lbFf[1] + hy, Tz = k.lbFf[2] + hz;
  const float hinv = 0.5f * inv;
  ux = __fmaf_rn(Tx, hinv, ux);
  uy = __fmaf_rn(Ty, hinv, uy);
  uz = __fmaf_rn(Tz, hinv, uz);
  const float usq = __fmaf_rn(ux, ux, __fmaf_rn(uy, uy, uz * uz));
  const float uT = __fmaf_rn(ux, Tx, __fmaf_rn(uy, Ty, uz * Tz));
  const float om = k.omegaF, omf = k.omegafF;
  const float omc = 1.0f - om;
  const float base = __fmaf_rn(-1.5f * n, usq, dr);  // dr - 1.5 n u^2
  // g' = (1 - om) g + om geq + omf guo with
  //   geq = w (dr + n (3 vu + 4.5 vu^2 - 1.5 u^2)),  guo = w (9 vu c.T + 3 (c.T - u.T)),
  // split into the part even in c (S) and the part odd in c (A), so that
  // g'_j = (1 - om) g_j + S + A and g'_opp = (1 - om) g_opp + S - A.
  const float a0s = om * base - omf * 3.0f * uT;
  const float a1s = om * 4.5f * n, a2s = omf * 9.0f, b1s = om * 3.0f * n, b2s = omf * 3.0f;
  g[0] = __fmaf_rn(omc, g[0], (float)WJ(0) * a0s);
#pragma unroll
  for (int j = 1; j < Q; j += 2) {
    const float w = (float)WJ(j);
    const float vu = dotcf(j, ux, uy, uz);
    const float cT = dotcf(j, Tx, Ty, Tz);
    const float S = w * __fmaf_rn(vu, __fmaf_rn(a1s, vu, a2s * cT), a0s);
    const float A = w * __fmaf_rn(b1s, vu, b2s * cT);
    g[j] = __fmaf_rn(omc, g[j], S + A);
    g[j + 1] = __fmaf_rn(omc, g[j + 1], S - A);
  }
  s.n = n;
  s.ux = ux;
  s.uy = uy;
  s.uz = uz;
  s.hx = hx;
  s.hy = hy;
  s.hz = hz;
}

}  // namespace lbdem
