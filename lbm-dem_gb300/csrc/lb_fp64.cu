// Plain FP64 lattice kernels: fused reconstruct / particle forcing /
// BGK+Guo collision / push streaming with bounce-back and the free-surface
// gas rule, the free-surface mass update and interface conversion, the
// impactor uncover/voxelisation and the particle flagging of the coupling
// step, and device-side initialisation.
//
// Arithmetic follows the reference operation by operation (no FMA
// contraction: this file is compiled with --fmad=false), so that each node
// update is bit-identical to the reference given identical inputs; only the
// order of the reductions (forces on particles, walls and the impactor, mass
// surpluses) differs. Terms with a zero lattice-velocity component are
// skipped; in the reference they add an exact +-0 (src/node.cpp:65,86,108,200).
//
// Reference functions restated here (paths relative to the reference root):
//   node::reconstruct/shiftVelocity/computeEquilibrium/solveCollision/addForce
//     src/node.cpp:75-207; LB::reconstruction/collision src/LB.cpp:1261-1332
//   LB::computeHydroForces src/LB.cpp:1901-1978
//   LB::streaming src/LB.cpp:1334-1544; LB::redistributeMass :1844-1852
//   LB::updateMass :1548-1639; LB::updateInterface :1641-1842
//   LB::updateObjectBoundaries/findNewActiveObject :797-943
//   LB::updateIndices/initializeParticleBoundaries :1875-1899, 683-711
//   LB::findNewActive :1980-2029 (its loop-exiting break included)
//   LB::latticeBolzmannInit and helpers :340-398, 538-564, 713-795, 974-1096
#include <cfloat>
#include <climits>

#include "lattice_common.cuh"

namespace lbdem {

// Fused LB step over all nodes: reconstruct, particle forcing, collision,
// push streaming with the boundary rules of LB::streaming, and the per-node
// bookkeeping of cleanLists / updateMass (fluid part).
template <bool RHEO>
__device__ __forceinline__ void lbStepFp64Impl(const Consts& k, const LbArgs& a) {
  __shared__ double acc[ACC_N];
  __shared__ int sbox[6];
  __shared__ int snif;
  __shared__ unsigned snact;
  for (int i = threadIdx.x; i < ACC_N; i += blockDim.x) acc[i] = 0.0;
  if (threadIdx.x < 3) sbox[threadIdx.x] = INT_MAX;
  else if (threadIdx.x < 6) sbox[threadIdx.x] = -1;
  if (threadIdx.x == 0) {
    snif = 0;
    snact = 0;
  }
  __syncthreads();
  const long long N = k.N;
  const long long NP = k.NP;  // population plane stride
  const double* fin = (const double*)a.fin;
  double* fout = (double*)a.fout;
  const int lane = threadIdx.x & 31;
  const long long warpsPerBlock = blockDim.x >> 5;
  const long long gw = blockIdx.x * warpsPerBlock + (threadIdx.x >> 5);
  const long long stride = (long long)gridDim.x * warpsPerBlock * 32;
  const double sp[Q] = {k.initDensity * WJ(0),  k.initDensity * WJ(1),  k.initDensity * WJ(2),
                        k.initDensity * WJ(3),  k.initDensity * WJ(4),  k.initDensity * WJ(5),
                        k.initDensity * WJ(6),  k.initDensity * WJ(7),  k.initDensity * WJ(8),
                        k.initDensity * WJ(9),  k.initDensity * WJ(10), k.initDensity * WJ(11),
                        k.initDensity * WJ(12), k.initDensity * WJ(13), k.initDensity * WJ(14),
                        k.initDensity * WJ(15), k.initDensity * WJ(16), k.initDensity * WJ(17),
                        k.initDensity * WJ(18)};
  BBAcc bba;
  for (long long base = gw * 32; base < N; base += stride) {
    const long long x = base + lane;
    const bool valid = x < N;
    uint8_t m = valid ? a.mask[x] : (uint8_t)2;
    const int t = m & TYPE_MASK;
    const bool act = valid && isActiveT(t);
    // cleanLists (the active list now equals the active types) and the
    // neighbour cache, written back once the links are classified
    uint8_t nm = (uint8_t)(act ? ((m | ABIT) & ~BULK) : (m & ~(ABIT | BULK)));
    const bool bulk = (m & BULK) != 0;
    bool allAct = true;
    int key = -1;
    double pv[16];
    if (act) {
      int ix, iy, iz;
      coords(k, x, ix, iy, iz);
      double f[Q];
#pragma unroll
      for (int j = 0; j < Q; ++j) f[j] = fin[(long long)j * NP + x];
      const bool pf = (m & PFLAG) != 0;
      const uint32_t pid = pf ? a.solid[x] : 0u;
      const double massOld = a.mass[x];
      NodeState s;
      collideNode<RHEO>(k, f, pf, pid, a.pkd, a.pkd + 3 * k.nPart, a.pw1, k.nPart, massOld, ix,
                        iy, iz, s, RHEO ? k.visc + x : nullptr, true);
      if (pf && pid < (uint32_t)k.nPart) {
        key = (int)pid;
        pv[0] = s.dx * 1.0;
        pv[1] = s.dy * 1.0;
        pv[2] = s.dz * 1.0;
        pv[3] = (s.ry * s.dz - s.rz * s.dy) * 1.0;
        pv[4] = (s.rz * s.dx - s.rx * s.dz) * 1.0;
        pv[5] = (s.rx * s.dy - s.ry * s.dx) * 1.0;
        const double r3[3] = {s.rx, s.ry, s.rz}, d3[3] = {s.dx, s.dy, s.dz};
#pragma unroll
        for (int aa = 0; aa < 3; ++aa)
#pragma unroll
          for (int bb = 0; bb < 3; ++bb)
            pv[6 + 3 * aa + bb] = 1.0 * r3[aa] * k.uLength * d3[bb] * k.uForce;
        pv[15] = massOld;
      } else if (pf) {
        atomicOr(a.iscal + IS_ERROR, ERR_PARTICLE_INDEX);
      }
      // LB::streaming, push form: population j of this node goes to the
      // neighbour x+c_j when it is active; otherwise this node receives the
      // reference's boundary value in direction opp(j).
      fout[x] = f[0];
      const double usq = s.ux * s.ux + s.uy * s.uy + s.uz * s.uz;
      const unsigned wallN = boxWallLinks(k, ix, iy, iz);
#pragma unroll
      for (int j = 1; j < Q; ++j) {
        const long long lk = x + nbrOffset(k, j);
        const bool wl = (wallN >> j) & 1u;
        // a cached node's links are active or box walls (all of type k.wallType)
        const int tl = bulk ? (wl ? k.wallType : 0) : (a.mask[lk] & TYPE_MASK);
        const double fs = f[j];
        const long long dst = (long long)OPPJ(j) * NP + x;
        allAct = allAct && (isActiveT(tl) || wl);
        if (isActiveT(tl)) {
          fout[(long long)j * NP + lk] = fs;
        } else if (tl == 2) {
          const double vuj = dotc(j, s.ux, s.uy, s.uz);
          fout[dst] = -fs + WJ(j) * k.initDensity * (2.0 + 9.0 * (vuj * vuj) - 3.0 * usq);
        } else if (tl == 11) {
          fout[dst] = fs;
        } else if (tl == 5 || tl == 6) {
          // slip walls: bounce-back without a wall force (the wall velocity
          // is zero, BBi == 0); the diagonal links' slip rule is applied by
          // slipStash / slipApply once every node has streamed
          fout[dst] = fs;
        } else if (tl == 7 || tl == 8) {
          // wall velocity is zero: BBi == 0 for dynamic walls as well
          const double bb = 2.0 * (fs - sp[j]) - 0.0;
          const uint32_t w = a.solid[lk];
          if (w < (uint32_t)k.nWall) {
            if (CX(j)) bba.wall(acc, (int)w, 0, CX(j) > 0 ? bb : -bb);
            if (CY(j)) bba.wall(acc, (int)w, 1, CY(j) > 0 ? bb : -bb);
            if (CZ(j)) bba.wall(acc, (int)w, 2, CZ(j) > 0 ? bb : -bb);
          }
          fout[dst] = fs;
        } else if (tl == 12) {
          const int ov = a.objIdx[lk];
          const double* ob = a.obj + ov * OB_STRIDE;
          const bool stale = (a.mask[lk] & OSTALE) != 0;
          const double vx = stale ? 0.0 : ob[OB_X1] / k.uSpeed,
                       vy = stale ? 0.0 : ob[OB_X1 + 1] / k.uSpeed,
                       vz = stale ? 0.0 : ob[OB_X1 + 2] / k.uSpeed;
          const double BBi = 2.0 * 3.0 * s.n * WJ(j) * dotc(j, vx, vy, vz);
          const double bb = 2.0 * (fs - sp[j]) - BBi;
          const uint32_t so = a.solid[lk];
          if (so < (uint32_t)k.nObj) {
            const double* os = a.obj + so * OB_STRIDE;
            int lx, ly, lz;
            coords(k, lk, lx, ly, lz);
            const double Fx = CX(j) ? (CX(j) > 0 ? bb : -bb) : 0.0;
            const double Fy = CY(j) ? (CY(j) > 0 ? bb : -bb) : 0.0;
            const double Fz = CZ(j) ? (CZ(j) > 0 ? bb : -bb) : 0.0;
            const double rx = (double)lx - os[OB_X0] / k.uLength;
            const double ry = (double)ly - os[OB_X0 + 1] / k.uLength;
            const double rz = (double)lz - os[OB_X0 + 2] / k.uLength;
            if (CX(j)) bba.obj(acc, (int)so, 0, Fx);
            if (CY(j)) bba.obj(acc, (int)so, 1, Fy);
            if (CZ(j)) bba.obj(acc, (int)so, 2, Fz);
            bba.obj(acc, (int)so, 3, ry * Fz - rz * Fy);
            bba.obj(acc, (int)so, 4, rz * Fx - rx * Fz);
            bba.obj(acc, (int)so, 5, rx * Fy - ry * Fx);
          }
          fout[dst] = fs - BBi;
          bba.extra += BBi * massOld;
        } else {
          atomicOr(a.iscal + IS_ERROR, ERR_TYPE);
        }
      }
      if (t == 3) {
        appendInterface((uint32_t)x, a.ifList, a.iscal);
        a.rhoS[x] = s.n;
        a.uS[x] = s.ux;
        a.uS[N + x] = s.uy;
        a.uS[2 * N + x] = s.uz;
        a.hS[x] = s.hx;
        a.hS[N + x] = s.hy;
        a.hS[2 * N + x] = s.hz;
        atomicMin(&sbox[0], ix);
        atomicMin(&sbox[1], iy);
        atomicMin(&sbox[2], iz);
        atomicMax(&sbox[3], ix);
        atomicMax(&sbox[4], iy);
        atomicMax(&sbox[5], iz);
      } else if (k.freeSurface) {
        a.mass[x] = s.n;  // LB::updateMass, fluid nodes (src/LB.cpp:1631-1634)
      }
      if (allAct) nm |= BULK;
    }
    if (valid && nm != m) a.mask[x] = nm;
    const unsigned ifb = __ballot_sync(0xffffffffu, act && t == 3);
    if (lane == 0 && ifb) atomicAdd(&snif, __popc(ifb));
    const unsigned acb = __ballot_sync(0xffffffffu, act);
    if (lane == 0 && acb) atomicAdd(&snact, (unsigned)__popc(acb));
    warpParticleReduce(key, pv, a.pFHydro, a.pMHydro, a.pSHydro, a.pFluidVol, k.nPart);
  }
  bba.flush(acc);
  __syncthreads();
  for (int i = threadIdx.x; i < ACC_N; i += blockDim.x) {
    const double v = acc[i];
    if (v == 0.0) continue;
    if (i < ACC_OBJ) atomicAdd(a.wallF + (i / 3) * 12 + (i % 3), v);
    else if (i < ACC_EXTRA) {
      const int o = (i - ACC_OBJ) / 6, c = (i - ACC_OBJ) % 6;
      atomicAdd(a.obj + o * OB_STRIDE + (c < 3 ? OB_FHYDRO + c : OB_MHYDRO + c - 3), v);
    } else {
      atomicAddComp(a.scal + SC_EXTRA_MASS, a.scal + SC_EXTRA_MASS_LO, v);
    }
  }
  if (threadIdx.x == 0) {
    if (snact) atomicAdd(a.uscal + US_ACTIVE_UPDATES, (unsigned long long)snact);
    if (snif) atomicAdd(a.iscal + IS_NIF, snif);
    if (sbox[3] >= 0) {
      atomicMin(a.iscal + IS_BBOX + 0, sbox[0]);
      atomicMin(a.iscal + IS_BBOX + 1, sbox[1]);
      atomicMin(a.iscal + IS_BBOX + 2, sbox[2]);
      atomicMax(a.iscal + IS_BBOX + 3, sbox[3]);
      atomicMax(a.iscal + IS_BBOX + 4, sbox[4]);
      atomicMax(a.iscal + IS_BBOX + 5, sbox[5]);
    }
  }
}

LBDEM_KERNEL(__launch_bounds__(256), lbStepFp64, LbArgs, lb) { lbStepFp64Impl<false>(k, a); }
// the same step with a per-node viscosity (non-Newtonian rheology or the
// Smagorinsky term, LB::collision src/LB.cpp:1322-1325)
LBDEM_KERNEL(__launch_bounds__(256), lbStepFp64Rheo, LbArgs, lb) { lbStepFp64Impl<true>(k, a); }

// Start of the LB step: the per-step reductions are cleared (particle
// sums, the float sums of the mixed form, impactor and wall hydrodynamic
// forces, extra mass, interface count and box) and the particle kinematics
// in lattice units are formed once per particle (x0/L, x1/S, w1/W: the
// quotients the reference forms at every node).
__device__ __forceinline__ void lbPrepareBody(const Consts& k, double* pAcc, long long pAccLen,
                                              float* pAccF, long long pAccFLen, double* obj,
                                              double* wallF, double* scal, int* iscal,
                                              const double* px0, const double* px1,
                                              const double* pw1, double* pkd, float* pkf) {
  const long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = i0; i < pAccLen; i += stride) pAcc[i] = 0.0;
  if (pAccF)
    for (long long i = i0; i < pAccFLen; i += stride) pAccF[i] = 0.0f;
  const int P = k.nPart;
  if (pkf) {
    // mixed form: [P] x (x0/L, x1/S, w1/W) as three float4 (4th lane 0), by
    // FP32 products with the reciprocal units (an FP64 division per value
    // costs more than the rest of the kernel); the FP64 copy is not used
    for (long long i = i0; i < 3LL * P; i += stride) {
      const long long p = i % P, c = i / P;
      pkf[12 * p + c] = (float)px0[i] * k.invLengthF;
      pkf[12 * p + 4 + c] = (float)px1[i] * k.invSpeedF;
      pkf[12 * p + 8 + c] = (float)pw1[i] * k.invAngVelF;
    }
  } else {
    for (long long i = i0; i < 3LL * P; i += stride) {
      pkd[i] = px0[i] / k.uLength;
      pkd[3 * P + i] = px1[i] / k.uSpeed;
    }
  }
  if (i0 < k.nObj) {
    for (int c = 0; c < 3; ++c) {
      obj[i0 * OB_STRIDE + OB_FHYDRO + c] = 0.0;
      obj[i0 * OB_STRIDE + OB_MHYDRO + c] = 0.0;
    }
  }
  if (i0 < k.nWall)
    for (int c = 0; c < 3; ++c) wallF[i0 * 12 + c] = 0.0;
  if (i0 == 0) {
    scal[SC_EXTRA_MASS] = 0.0;
    scal[SC_EXTRA_MASS_LO] = 0.0;
    iscal[IS_NIF] = 0;
    iscal[IS_IFLIST] = 0;
    iscal[IS_BBOX + 0] = iscal[IS_BBOX + 1] = iscal[IS_BBOX + 2] = INT_MAX;
    iscal[IS_BBOX + 3] = iscal[IS_BBOX + 4] = iscal[IS_BBOX + 5] = -1;
  }
}

// A node of the lattice's outer layer (the box walls). An impactor that
// reaches the walls turns wall nodes into impactor nodes (as the reference
// does); once uncovered, such a node becomes gas whatever its neighbours,
// since an active node there would stream beyond the lattice (the
// reference's neighbour offsets leave the node array there too).
__device__ __forceinline__ bool onOuterLayer(const Consts& k, int ix, int iy, int iz) {
  return ix == 0 || iy == 0 || iz == 0 || ix == k.X - 1 || iy == k.Y - 1 || iz == k.Z - 1;
}

__device__ __forceinline__ bool fsRegion(const Consts& k, const int* iscal, int& x0, int& y0,
                                         int& z0, int& rx, int& ry, int& rz) {
  if (iscal[IS_BBOX + 3] < 0) return false;
  x0 = max(iscal[IS_BBOX + 0] - 1, 0);
  y0 = max(iscal[IS_BBOX + 1] - 1, 0);
  z0 = max(iscal[IS_BBOX + 2] - 1, 0);
  rx = min(iscal[IS_BBOX + 3] + 1, k.X - 1) - x0 + 1;
  ry = min(iscal[IS_BBOX + 4] + 1, k.Y - 1) - y0 + 1;
  rz = min(iscal[IS_BBOX + 5] + 1, k.Z - 1) - z0 + 1;
  return true;
}

// Walk of a box of rx x ry nodes per layer by a grid-stride loop: the
// box coordinates of linear index i are carried from one iteration to the
// next by the stride's own decomposition (no division per node).
struct BoxWalk {
  unsigned bx, by, bz, sx, sy, sz;
  __device__ __forceinline__ BoxWalk(unsigned i, unsigned stride, unsigned rx, unsigned ry) {
    bx = i % rx;
    by = (i / rx) % ry;
    bz = i / (rx * ry);
    sx = stride % rx;
    sy = (stride / rx) % ry;
    sz = stride / (rx * ry);
  }
  __device__ __forceinline__ void next(unsigned rx, unsigned ry) {
    bx += sx;
    by += sy;
    bz += sz;
    if (bx >= rx) {
      bx -= rx;
      ++by;
    }
    if (by >= ry) {
      by -= ry;
      ++bz;
    }
  }
};

// Grid-stride loop over the region's nodes (ix, iy, iz, x); boxes lie in
// the lattice, so their volumes fit 32 bits as node indices do.
#define FS_LOOP(k, a, ...)                                                               \
  int _x0, _y0, _z0, _rx, _ry, _rz;                                                      \
  if (fsRegion(k, a.iscal, _x0, _y0, _z0, _rx, _ry, _rz)) {                              \
    const unsigned _vol = (unsigned)_rx * (unsigned)_ry * (unsigned)_rz;                 \
    const unsigned _stride = gridDim.x * blockDim.x;                                     \
    unsigned _i = blockIdx.x * blockDim.x + threadIdx.x;                                 \
    BoxWalk _w(_i, _stride, (unsigned)_rx, (unsigned)_ry);                               \
    for (; _i < _vol; _i += _stride, _w.next((unsigned)_rx, (unsigned)_ry)) {            \
      const int ix = _x0 + (int)_w.bx;                                                   \
      const int iy = _y0 + (int)_w.by;                                                   \
      const int iz = _z0 + (int)_w.bz;                                                   \
      const long long x = ix + iy * k.sy + iz * k.sz;                                    \
      __VA_ARGS__                                                                        \
    }                                                                                    \
  }

// Unit conversions at the end of LB::streaming / computeHydroForces and the
// mass-redistribution amount (src/LB.cpp:1533-1543, 1966-1977, 1844-1847).
__device__ __forceinline__ void lbFinalizeBody(const Consts& k, double* pF, double* pM,
                                               double* pV, double* obj, double* wallF,
                                               double* scal, const int* iscal,
                                               const float* pAccF, double* pS,
                                               const FsArgs& fa, int redistribute) {
  // the redistribution amount, once per block (an FP64 division in every
  // thread costs more than the rest of the kernel), formed first so that its
  // latency overlaps the particle conversions
  __shared__ double sAddMass;
  if (threadIdx.x == 0)
    sAddMass = (scal[SC_EXTRA_MASS] + scal[SC_EXTRA_MASS_LO]) / (double)(unsigned)iscal[IS_NIF];
  const int P = k.nPart;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    if (pAccF) {
      // mixed form: float sums [P][ACCF_STRIDE] of d (3), R_ab = sum r_a d_b
      // (9) and massOld (1); torque = antisymmetric part of R, stresslet = R
      // in physical units (src/LB.cpp:1941-1958). The unit products are
      // taken in FP32, the precision of the sums, and stored as FP64.
      const float4* a4 = reinterpret_cast<const float4*>(pAccF + (size_t)i * ACCF_STRIDE);
      const float4 q0 = a4[0], q1 = a4[1], q2 = a4[2], q3 = a4[3];
      const float R[9] = {q0.w, q1.x, q1.y, q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
      pF[i] = (double)(q0.x * k.uForceF);
      pF[P + i] = (double)(q0.y * k.uForceF);
      pF[2 * P + i] = (double)(q0.z * k.uForceF);
      pM[i] = (double)((R[5] - R[7]) * k.uTorqueF);
      pM[P + i] = (double)((R[6] - R[2]) * k.uTorqueF);
      pM[2 * P + i] = (double)((R[1] - R[3]) * k.uTorqueF);
      for (int c = 0; c < 9; ++c) pS[c * P + i] = (double)(R[c] * k.sLF);
      pV[i] = (double)(q3.x * k.uVolumeF);
      continue;
    }
    for (int c = 0; c < 3; ++c) {
      pF[c * P + i] *= k.uForce;
      pM[c * P + i] *= k.uTorque;
    }
    pV[i] *= k.uVolume;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // (the mixed form's wall-force sweep adds its sums in physical units)
    if (!k.mixed)
      for (int w = 0; w < k.nWall; ++w)
        for (int c = 0; c < 3; ++c) wallF[w * 12 + c] *= k.uForce;
    for (int o = 0; o < k.nObj; ++o)
      for (int c = 0; c < 3; ++c) {
        obj[o * OB_STRIDE + OB_FHYDRO + c] *= k.uForce;
        obj[o * OB_STRIDE + OB_MHYDRO + c] *= k.uTorque;
      }
    scal[SC_ADD_MASS] = sAddMass;
  }
  if (redistribute) {
    // LB::redistributeMass(extraMass) over the interface nodes
    __syncthreads();
    const double addMass = sAddMass;
    const int nl = fa.iscal[IS_IFLIST];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nl; i += gridDim.x * blockDim.x) {
      const uint32_t x = fa.ifList[i];
      // the mass the collision used, for fsUpdateMass's recomputation
      fa.massNew[x] = fa.mass[x];
      fa.mass[x] += addMass;
    }
  }
}

// ---- free surface ----------------------------------------------------------


enum : uint8_t { FS_FILLED = 1, FS_EMPTIED = 2, FS_NEW = 4 };

// Region = interface bounding box of the LB step grown by one node.
// dst += the block's sum of v; with lo, compensated (atomicAddComp)
// with any = whether this thread added anything to v; a block where no
// thread did adds nothing and skips the FP64 reduction (same result: the
// sum of zeros is not added either)
__device__ __forceinline__ void blockAddDouble(double v, bool any, double* dst,
                                               double* lo = nullptr) {
  if (!__syncthreads_or(any)) return;
  __shared__ double red[32];
  const unsigned FULL = 0xffffffffu;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    double s = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    if (l == 0 && s != 0.0) {
      if (lo) atomicAddComp(dst, lo, s);
      else atomicAdd(dst, s);
    }
  }
  __syncthreads();
}


// Post-collision populations of interface node x (deviations in the mixed
// form), recomputed from its pre-collision populations for the links into
// walls and impactors. Kept out of line: few nodes need it, and inlined it
// would set the register count of the whole mass update.
__device__ __noinline__ void fsPostCollision(const Consts& k, const FsArgs& a, long long x,
                                             uint8_t m, int ix, int iy, int iz, double* fsl) {
  const bool pf = (m & PFLAG) != 0;
  if (k.mixed) {
    float g[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) g[q] = ((const float*)a.fold)[(long long)q * k.NP + x];
    NodeStateF s;
    const uint32_t pid = pf ? a.solid[x] : 0u;
    const bool coupled = pf && pid < (uint32_t)k.nPart;
    const KinF kin = coupled ? loadKinF(a.pkf, pid) : KinF{};
    collideNodeMixed(k, g, coupled, kin, (float)a.massNew[x], ix, iy, iz, s);
#pragma unroll
    for (int q = 0; q < Q; ++q) fsl[q] = (double)g[q];
  } else {
#pragma unroll
    for (int q = 0; q < Q; ++q) fsl[q] = ((const double*)a.fold)[(long long)q * k.NP + x];
    NodeState s;
    // with a per-node viscosity, the one the lattice step's collision used
    // (and stored) is used again
    if (k.visc)
      collideNode<true>(k, fsl, pf, pf ? a.solid[x] : 0u, a.pkd, a.pkd + 3 * k.nPart, a.pw1,
                        k.nPart, a.massNew[x], ix, iy, iz, s, k.visc + x, false);
    else
      collideNode(k, fsl, pf, pf ? a.solid[x] : 0u, a.pkd, a.pkd + 3 * k.nPart, a.pw1, k.nPart,
                  a.massNew[x], ix, iy, iz, s);
  }
}

// slip-wall tables and partner lookup (LB::streaming and LB::updateMass,
// src/LB.cpp:1454-1523, 1595-1625; src/lattice.h:137-140); see slipPass
__constant__ unsigned char c_slip1Check[Q] = {0, 0, 0, 0, 0, 0, 0, 1, 2, 3, 4, 3, 4, 5, 6, 1, 2, 6, 5};
__constant__ unsigned char c_slip1[Q] = {0, 0, 0, 0, 0, 0, 0, 9, 10, 8, 7, 13, 14, 12, 11, 18, 17, 15, 16};
__constant__ unsigned char c_slip2Check[Q] = {0, 0, 0, 0, 0, 0, 0, 3, 4, 2, 1, 5, 6, 4, 3, 5, 6, 1, 2};
__constant__ unsigned char c_slip2[Q] = {0, 0, 0, 0, 0, 0, 0, 10, 9, 7, 8, 14, 13, 11, 12, 17, 18, 16, 15};

// the slip partner of link j of x: 1 or 2 when exactly that check node is
// active, 0 otherwise
__device__ __forceinline__ int slipPartner(const Consts& k, const uint8_t* mask, long long x,
                                           int j, long long& c, int& s) {
  const long long c1 = x + nbrOffset(k, c_slip1Check[j]);
  const long long c2 = x + nbrOffset(k, c_slip2Check[j]);
  const bool a1 = isActiveT(mask[c1] & TYPE_MASK), a2 = isActiveT(mask[c2] & TYPE_MASK);
  if (a1 && !a2) {
    c = c1;
    s = c_slip1[j];
    return 1;
  }
  if (!a1 && a2) {
    c = c2;
    s = c_slip2[j];
    return 2;
  }
  return 0;
}
__device__ __forceinline__ bool slipOneActive(const Consts& k, const uint8_t* mask, long long x,
                                              int j) {
  long long c;
  int s;
  return slipPartner(k, mask, x, j, c, s) != 0;
}

// The exchange sum of one interface node in FP64 (the plain form, and the
// mixed form's nodes with a wall or impactor link), in link order. Kept out
// of line so that the mixed form's FP32 path keeps few registers.
__device__ __noinline__ double fsMassDeltaFp64(const Consts& k, const FsArgs& a, long long x,
                                               uint8_t m, int ix, int iy, int iz, double mx,
                                               unsigned liq, unsigned ifc, unsigned wal,
                                               unsigned slp) {
  double fsl[Q];
  if (wal) fsPostCollision(k, a, x, m, ix, iy, iz, fsl);
  double delta = 0.0;
  bool first = true;
#pragma unroll
  for (int j = 1; j < Q; ++j) {
    double term;
    if ((liq >> j) & 1u) {
      const long long lk = x + nbrOffset(k, j);
      const double ms = fdiff(k, a.fcur, OPPJ(j), x, j, lk);
      term = ((ifc >> j) & 1u) ? 0.5 * (a.mass[lk] + mx) * ms : 1.0 * ms;
    } else if ((wal >> j) & 1u) {
      // f_opp(x) after streaming minus the population x sent into the wall
      const double ms = k.mixed
          ? (double)((const float*)a.fcur)[(long long)OPPJ(j) * k.NP + x] - fsl[j]
          : ((const double*)a.fcur)[(long long)OPPJ(j) * k.NP + x] - fsl[j];
      double w = 1.0;  // averageMass = w * mass (src/LB.cpp:1581-1625)
      if (((slp >> j) & 1u) && j > 6 && slipOneActive(k, a.mask, x, j)) w = 1.0 - k.slipS1;
      term = (w * mx) * ms;
    } else {
      continue;
    }
    delta = first ? term : delta + term;
    first = false;
  }
  return delta;
}

// LB::updateMass (interface part). The neighbour types are read first, all
// links at once; the mass exchange terms are then summed in link order.
LBDEM_KERNEL(__launch_bounds__(256, 2), fsUpdateMass, FsArgs, fs) {
  // the free-surface step's surplus and interface count start from zero
  // (fsUpdateMass itself accumulates neither)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.scal[SC_SURPLUS] = 0.0;
    a.scal[SC_SURPLUS_LO] = 0.0;
    a.iscal[IS_NIF2] = 0;
  }
  // over the interface nodes the lattice step listed (none has changed
  // type since)
  const int nl = a.iscal[IS_IFLIST];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nl; i += gridDim.x * blockDim.x) {
    const long long x = a.ifList[i];
    const uint8_t m = a.mask[x];
    int ix, iy, iz;
    coords(k, x, ix, iy, iz);
    const double mx = a.mass[x];
    // links to fluid or interface nodes, to interface nodes, to walls/impactors
    unsigned liq = 0, ifc = 0, wal = 0, slp = 0;
#pragma unroll
    for (int j = 1; j < Q; ++j) {
      const int tl = a.mask[x + nbrOffset(k, j)] & TYPE_MASK;
      liq |= (unsigned)(tl == 3 || tl == 0) << j;
      ifc |= (unsigned)(tl == 3) << j;
      wal |= (unsigned)(tl == 8 || tl == 12 || tl == 9) << j;
      slp |= (unsigned)(tl == 6) << j;  // moving slip wall (a static one adds no mass)
    }
    wal |= slp;
    if (k.mixed && !wal) {
      // mixed form, no wall or impactor link: the exchange terms from the
      // FP32 deviations in FP32 (f_opp(x) - f_j(x + c_j) = g_opp - g_j, the
      // weights cancel), summed in link order, added to the FP64 mass once.
      // Each term is the exact negative of the neighbour's term for the same
      // link, as in FP64; only the per-node sum rounds in FP32.
      const float* F = (const float*)a.fcur;
      const size_t NP = (size_t)k.NP;
      const float mxf = (float)mx;
      float dl = 0.0f;
#pragma unroll
      for (int j = 1; j < Q; ++j) {
        if (!((liq >> j) & 1u)) continue;
        const long long lk = x + nbrOffset(k, j);
        const float ms = F[OPPJ(j) * NP + x] - F[j * NP + lk];
        dl += ((ifc >> j) & 1u) ? (0.5f * ((float)a.mass[lk] + mxf)) * ms : ms;
      }
      a.massNew[x] = mx + (double)dl;
      continue;
    }
    a.massNew[x] = mx + fsMassDeltaFp64(k, a, x, m, ix, iy, iz, mx, liq, ifc, wal, slp);
  }
}

// findInterfaceMutants (src/LB.cpp:1669-1698) after the interface mass copy.
LBDEM_KERNEL(, fsMutants, FsArgs, fs) {
  FS_LOOP(k, a, {
    const uint8_t m = a.mask[x];
    a.fsflag[x] = 0;
    if ((m & TYPE_MASK) != 3) continue;
    const double mm = a.massNew[x];
    a.mass[x] = mm;
    if (mm > a.rhoS[x]) {
      a.mask[x] = (uint8_t)((m & ~TYPE_MASK) | 0);
      a.fsflag[x] = FS_FILLED;
    } else if (mm < 0.0) {
      a.mask[x] = (uint8_t)((m & ~TYPE_MASK) | 2);
      a.fsflag[x] = FS_EMPTIED;
    }
  })
}

// smoothenInterface (src/LB.cpp:1700-1749): gas neighbours of filled nodes
// become interface nodes initialised from the first filled neighbour in the
// reference's order (the highest node index); fluid neighbours of emptied
// nodes become interface nodes holding 99% of their density.
LBDEM_KERNEL(, fsSmoothen, FsArgs, fs) {
  double surplus = 0.0;
  bool touched = false;
  FS_LOOP(k, a, {
    const uint8_t m = a.mask[x];
    const int t = m & TYPE_MASK;
    // a gas node of the outer layer (an uncovered wall node) stays gas: its
    // links leave the lattice
    if (t == 2 && !onOuterLayer(k, ix, iy, iz)) {
      long long win = -1;
#pragma unroll 1
      for (int j = 1; j < Q; ++j) {
        const long long lk = x + nbrOffset(k, j);
        if ((a.fsflag[lk] & FS_FILLED) && lk > win) win = lk;
      }
      if (win >= 0) {
        const double rho0 = k.initDensity;
        const double Fx = a.hS[win] + k.lbF[0], Fy = a.hS[k.N + win] + k.lbF[1],
                     Fz = a.hS[2 * k.N + win] + k.lbF[2];
        const double ux = Fx / 2.0 / rho0 + a.uS[win];
        const double uy = Fy / 2.0 / rho0 + a.uS[k.N + win];
        const double uz = Fz / 2.0 / rho0 + a.uS[2 * k.N + win];
        const double usq = ux * ux + uy * uy + uz * uz;
#pragma unroll
        for (int j = 0; j < Q; ++j) fset(k, a.fcur, j, x, feqj(j, rho0, ux, uy, uz, usq));
        a.mask[x] = (uint8_t)((m & ~TYPE_MASK) | 3);
        markActive(k, x);
        a.fsflag[x] |= FS_NEW;
        a.rhoS[x] = rho0;
        a.mass[x] = 0.01 * rho0;
        if (k.visc) k.visc[x] = k.visc[win];  // the filler's viscosity (src/LB.cpp:1719)
        surplus -= 0.01 * rho0;
        touched = true;
      }
    } else if (t == 0) {
      bool hit = false;
#pragma unroll 1
      for (int j = 1; j < Q; ++j)
        if (a.fsflag[x + nbrOffset(k, j)] & FS_EMPTIED) {
          hit = true;
          break;
        }
      if (hit) {
        const double n = (a.fsflag[x] & FS_FILLED) ? a.rhoS[x]
                       : (k.mixed ? (double)a.nF[x] : a.mass[x]);
        a.mask[x] = (uint8_t)((m & ~TYPE_MASK) | 3);
        a.fsflag[x] |= FS_NEW;
        a.rhoS[x] = n;
        a.mass[x] = 0.99 * n;
        surplus += 0.01 * n;
        touched = true;
      }
    }
  })
  blockAddDouble(surplus, touched, a.scal + SC_SURPLUS, a.scal + SC_SURPLUS_LO);
}

// updateMutants + removeIsolated, first pass (src/LB.cpp:1751-1817).
LBDEM_KERNEL(, fsMutantsAndFill, FsArgs, fs) {
  double surplus = 0.0;
  bool touched = false;
  FS_LOOP(k, a, {
    const uint8_t fl = a.fsflag[x];
    const uint8_t m = a.mask[x];
    if ((fl & FS_EMPTIED) && !(fl & FS_NEW)) {
      surplus += a.mass[x];
      a.mass[x] = 0.0;
      touched = true;
    } else if ((fl & FS_FILLED) && !(fl & FS_NEW)) {
      surplus += a.mass[x] - a.rhoS[x];
      touched = true;
      a.mass[x] = a.rhoS[x];
      if (k.mixed) a.nF[x] = (float)a.rhoS[x];
    } else if ((m & TYPE_MASK) == 3) {
      bool gasNb = false;
#pragma unroll 1
      for (int j = 1; j < Q; ++j)
        if ((a.mask[x + nbrOffset(k, j)] & TYPE_MASK) == 2) {
          gasNb = true;
          break;
        }
      if (!gasNb) {
        surplus += a.mass[x] - a.rhoS[x];
        touched = true;
        a.mass[x] = a.rhoS[x];
        if (k.mixed) a.nF[x] = (float)a.rhoS[x];
        a.mask[x] = (uint8_t)((m & ~TYPE_MASK) | 0);
      }
    }
  })
  blockAddDouble(surplus, touched, a.scal + SC_SURPLUS, a.scal + SC_SURPLUS_LO);
}

// removeIsolated, second pass (src/LB.cpp:1819-1841), and the interface count.
LBDEM_KERNEL(, fsEmptyIsolated, FsArgs, fs) {
  double surplus = 0.0;
  bool touched = false;
  int cnt = 0;
  FS_LOOP(k, a, {
    const uint8_t m = a.mask[x];
    if ((m & TYPE_MASK) != 3) continue;
    bool fluidNb = false;
#pragma unroll 1
    for (int j = 1; j < Q; ++j)
      if ((a.mask[x + nbrOffset(k, j)] & TYPE_MASK) == 0) {
        fluidNb = true;
        break;
      }
    if (!fluidNb) {
      surplus += a.mass[x];
      touched = true;
      a.mass[x] = 0.0;
      a.mask[x] = (uint8_t)((m & ~TYPE_MASK) | 2);
    } else {
      ++cnt;
    }
  })
  blockAddDouble(surplus, touched, a.scal + SC_SURPLUS, a.scal + SC_SURPLUS_LO);
  if (cnt) atomicAdd(a.iscal + IS_NIF2, cnt);
}

// redistributeMass(massSurplus) + cleanLists of the free-surface step over
// the interface box grown by 1, and the neighbour-cache upkeep over the box
// grown by 2: the nodes that left the active types in this step (interface
// -> gas) lie in the box grown by 1, so their neighbours lie in the box
// grown by 2. Every thread writes only its own node's mask byte.
LBDEM_KERNEL(, fsRedistribute, FsArgs, fs) {
  // the quotient once per block (an FP64 division in every thread costs
  // more than the rest of the kernel)
  __shared__ double sAddMass;
  if (threadIdx.x == 0)
    sAddMass = (a.scal[SC_SURPLUS] + a.scal[SC_SURPLUS_LO]) / (double)(unsigned)a.iscal[IS_NIF2];
  __syncthreads();
  const double addMass = sAddMass;
  int x1, y1, z1, rx1, ry1, rz1;
  if (!fsRegion(k, a.iscal, x1, y1, z1, rx1, ry1, rz1)) return;
  const int x0 = max(a.iscal[IS_BBOX + 0] - 2, 0), y0 = max(a.iscal[IS_BBOX + 1] - 2, 0),
            z0 = max(a.iscal[IS_BBOX + 2] - 2, 0);
  const unsigned rx = min(a.iscal[IS_BBOX + 3] + 2, k.X - 1) - x0 + 1,
                 ry = min(a.iscal[IS_BBOX + 4] + 2, k.Y - 1) - y0 + 1,
                 rz = min(a.iscal[IS_BBOX + 5] + 2, k.Z - 1) - z0 + 1;
  const unsigned vol = rx * ry * rz;
  const unsigned stride = gridDim.x * blockDim.x;
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  BoxWalk bw(i, stride, rx, ry);
  for (; i < vol; i += stride, bw.next(rx, ry)) {
    const int ix = x0 + (int)bw.bx, iy = y0 + (int)bw.by, iz = z0 + (int)bw.bz;
    const long long x = ix + iy * k.sy + iz * k.sz;
    const uint8_t m = a.mask[x];
    uint8_t nm = (uint8_t)(m & ~BULK);
    if (ix >= x1 && ix < x1 + rx1 && iy >= y1 && iy < y1 + ry1 && iz >= z1 && iz < z1 + rz1) {
      const int t = m & TYPE_MASK;
      if (t == 3) a.mass[x] += addMass;
      nm = (uint8_t)(isActiveT(t) ? (nm | ABIT) : (nm & ~ABIT));
      a.fsflag[x] = 0;
    }
    if (nm != m) a.mask[x] = nm;
  }
}

// ---- coupling step -----------------------------------------------------------

// Bounding box of the nodes inside a sphere (lattice units), clamped.
__device__ __forceinline__ void sphereBox(const Consts& k, double cx, double cy, double cz,
                                          double r, int* lo, int* hi) {
  const double c[3] = {cx, cy, cz};
  const int lim[3] = {k.X, k.Y, k.Z};
  // clamped in double before the conversion, so that a sphere of a diverged
  // run (a coordinate beyond the int range, or NaN) gets an empty box
  for (int a = 0; a < 3; ++a) {
    const double l = floor(c[a] - r) - 1.0, h = ceil(c[a] + r) + 1.0;
    if (!(l <= h)) {
      lo[a] = 0;
      hi[a] = -1;
      continue;
    }
    lo[a] = (int)fmin(fmax(l, 0.0), (double)lim[a]);
    hi[a] = (int)fmin(fmax(h, -1.0), (double)(lim[a] - 1));
  }
}

// One impactor in lattice units (the quotients the reference forms at every
// node, formed once per block) with its node box.
struct SphereL {
  double c[3], r;
  int lo[3], hi[3];
  SphereBoxTest t;  // the FP32 test relative to lo, FP64 near the surface
};
// threads 0 .. nObj-1 fill s[] from the records' position at offset xoff
// (OB_X0 or OB_X0PREV); the caller synchronises the block afterwards
__device__ __forceinline__ void loadSpheres(const Consts& k, const double* obj, int xoff,
                                            SphereL* s) {
  const int o = threadIdx.x;
  if (o < k.nObj) {
    const double* ob = obj + o * OB_STRIDE;
    for (int a = 0; a < 3; ++a) s[o].c[a] = ob[xoff + a] / k.uLength;
    s[o].r = ob[OB_R] / k.uLength;
    sphereBox(k, s[o].c[0], s[o].c[1], s[o].c[2], s[o].r, s[o].lo, s[o].hi);
    s[o].t = sphereBoxTest(s[o].c[0], s[o].c[1], s[o].c[2], s[o].r, s[o].lo);
  }
}

// findNewActiveObject, step 1: collect the nodes of LB::objectNodes that
// object 0 no longer covers. objectNodes (src/LB.cpp:770-789, 822-839) holds
// the object nodes that lay inside the sphere of the object their solid
// index names, at that object's position of the previous voxelisation; an
// object node outside it (one a restart file typed) is never uncovered.
__device__ __forceinline__ void uncoverCollectBody(const Consts& k, const uint8_t* mask,
                                                   const uint32_t* solid, const double* obj,
                                                   uint32_t* list, int* iscal) {
  __shared__ SphereL cur[MAX_OBJ], prev[MAX_OBJ];
  loadSpheres(k, obj, OB_X0, cur);
  loadSpheres(k, obj, OB_X0PREV, prev);
  __syncthreads();
  for (int o = 0; o < k.nObj; ++o) {
    const int* lo = prev[o].lo;
    const int* hi = prev[o].hi;
    if (hi[0] < lo[0] || hi[1] < lo[1] || hi[2] < lo[2]) continue;
    // a box within the lattice: its volume fits 32 bits, as node indices do
    const unsigned nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    const unsigned vol = nx * ny * nz;
    const unsigned stride = gridDim.x * blockDim.x;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    BoxWalk bw(i, stride, nx, ny);
    for (; i < vol; i += stride, bw.next(nx, ny)) {
      const int ix = lo[0] + (int)bw.bx, iy = lo[1] + (int)bw.by, iz = lo[2] + (int)bw.bz;
      const long long x = ix + iy * k.sy + iz * k.sz;
      if ((mask[x] & TYPE_MASK) != 12) continue;
      // member of objectNodes: inside its own object's previous sphere
      if (solid[x] != (uint32_t)o || !insideBox(prev[o].t, ix, iy, iz)) continue;
      if (insideBox(cur[0].t, ix, iy, iz)) continue;
      const int slot = atomicAdd(iscal + IS_NUNCOVER, 1);
      if (slot < UNCOVER_CAP) list[slot] = (uint32_t)x;
      else atomicOr(iscal + IS_ERROR, ERR_UNCOVER_CAP);
    }
  }
}

// Named barrier 1 over the first nthreads threads of the block (a multiple
// of 32), and the same barrier returning whether v was non-zero in any of
// them (the non-aligned forms: a warp may arrive with its lanes diverged).
__device__ __forceinline__ void teamSync(int nthreads) {
  asm volatile("barrier.sync 1, %0;" ::"r"(nthreads) : "memory");
}
__device__ __forceinline__ int teamOr(int nthreads, int v) {
  int r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n"
      " barrier.red.or.pred q, 1, %2, p;\n selp.s32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"(v), "r"(nthreads)
      : "memory");
  return r;
}

// uncoverResolve for n <= 32 H candidates of one impactor, by one warp:
// lane l holds candidates l and, for H = 2, l + 32 (after a shuffle bitonic
// sort, ascending node index). Each candidate records which lower-index
// candidates are its neighbours (a bit mask over the 32 H positions) and the
// fixed types of its other neighbours; the fixed-point iteration then takes
// two ballots per half per round. Results go to s_idx / s_st (bits 0-3 the
// new type) for the block's initialisation.
template <int H>
__device__ __forceinline__ void uncoverResolveWarp(const Consts& k, const uint8_t* mask,
                                                   const uint32_t* list, int n, uint32_t* s_idx,
                                                   uint8_t* s_st, int* s_n) {
  const unsigned FULLM = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  uint32_t x[H];
#pragma unroll
  for (int h = 0; h < H; ++h) x[h] = 32 * h + lane < n ? list[32 * h + lane] : 0xffffffffu;
  // bitonic sort of the 32 H keys, key e = 32 h + lane ascending
#pragma unroll
  for (int size = 2; size <= 32 * H; size <<= 1)
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride == 32) {  // (H = 2) the partner is the lane's other key
        const bool up = (lane & size) == 0;
        const uint32_t lo = min(x[0], x[H - 1]), hi = max(x[0], x[H - 1]);
        x[0] = up ? lo : hi;
        x[H - 1] = up ? hi : lo;
      } else {
#pragma unroll
        for (int h = 0; h < H; ++h) {
          const int e = 32 * h + lane;
          const uint32_t other = __shfl_xor_sync(FULLM, x[h], stride);
          const bool up = (e & size) == 0, low = (e & stride) == 0;
          x[h] = (low == up) ? min(x[h], other) : max(x[h], other);
        }
      }
    }
  bool valid[H], edge[H];
  uint32_t lk[H][Q];
  unsigned inb[H];
#pragma unroll
  for (int h = 0; h < H; ++h) {
    valid[h] = 32 * h + lane < n;
    int ix = 0, iy = 0, iz = 0;
    if (valid[h]) coords(k, (long long)x[h], ix, iy, iz);
    edge[h] = onOuterLayer(k, ix, iy, iz);
    inb[h] = 0;
#pragma unroll
    for (int j = 1; j < Q; ++j) {
      const int tx = ix + CX(j), ty = iy + CY(j), tz = iz + CZ(j);
      const bool in =
          valid[h] && tx >= 0 && tx < k.X && ty >= 0 && ty < k.Y && tz >= 0 && tz < k.Z;
      inb[h] |= (unsigned)in << j;
      lk[h][j] = in ? x[h] + (uint32_t)nbrOffset(k, j) : 0xffffffffu;
    }
  }
  // which links end on a candidate; lower candidates as a position mask
  unsigned candLinks[H];
  unsigned long long back[H];
#pragma unroll
  for (int h = 0; h < H; ++h) {
    candLinks[h] = 0;
    back[h] = 0;
  }
  for (int b = 0; b < n; ++b) {
    const uint32_t xb = __shfl_sync(FULLM, x[H == 2 && b >= 32 ? 1 : 0], b & 31);
#pragma unroll
    for (int h = 0; h < H; ++h)
#pragma unroll
      for (int j = 1; j < Q; ++j)
        if (lk[h][j] == xb) {
          candLinks[h] |= 1u << j;
          if (b < 32 * h + lane) back[h] |= 1ull << b;
        }
  }
  // the other neighbours' types (a higher candidate reads as an impactor node)
  bool fixFluid[H], fixGas[H];
#pragma unroll
  for (int h = 0; h < H; ++h) {
    uint8_t tls[Q];
#pragma unroll
    for (int j = 1; j < Q; ++j)
      tls[j] = ((inb[h] & ~candLinks[h]) >> j) & 1u ? (uint8_t)(mask[lk[h][j]] & TYPE_MASK)
                                                    : (uint8_t)0xFF;
    fixFluid[h] = fixGas[h] = false;
#pragma unroll
    for (int j = 1; j < Q; ++j) {
      fixFluid[h] |= tls[j] == 0;
      fixGas[h] |= tls[j] == 2;
    }
  }
  uint8_t st[H];  // 12: unresolved, neither fluid nor gas to its neighbours
#pragma unroll
  for (int h = 0; h < H; ++h) st[h] = 12;
  for (int it = 0; it <= n; ++it) {
    unsigned long long fluidL = 0, gasL = 0;
#pragma unroll
    for (int h = 0; h < H; ++h) {
      fluidL |= (unsigned long long)__ballot_sync(FULLM, valid[h] && st[h] == 0) << (32 * h);
      gasL |= (unsigned long long)__ballot_sync(FULLM, valid[h] && st[h] == 2) << (32 * h);
    }
    bool changed = false;
#pragma unroll
    for (int h = 0; h < H; ++h) {
      const bool fluidNb = fixFluid[h] || (back[h] & fluidL) != 0;
      const bool gasNb = fixGas[h] || (back[h] & gasL) != 0;
      const uint8_t nst = (!fluidNb || edge[h]) ? 2 : gasNb ? 3 : 0;
      changed |= valid[h] && nst != st[h];
      if (valid[h]) st[h] = nst;
    }
    if (!__any_sync(FULLM, changed)) break;
  }
#pragma unroll
  for (int h = 0; h < H; ++h)
    if (valid[h]) {
      s_idx[32 * h + lane] = x[h];
      s_st[32 * h + lane] = st[h];
    }
  if (lane == 0) *s_n = n;
}

// findNewActiveObject, step 2 (one CTA): resolve the uncovered nodes in the
// reference's serial order (ascending node index, each node seeing the new
// types of the lower-index ones) by fixed-point iteration, then initialise
// them (src/LB.cpp:874-940). Dynamic shared memory (UNCOVER_SMEM bytes):
// the sorted candidates, for each the indices of its lower-index candidate
// neighbours (at most the 9 links with a negative node offset), and its state.
__device__ __forceinline__ void uncoverResolveBody(const Consts& k, uint8_t* mask, void* f,
                                                   double* mass, float* nF, uint32_t* list,
                                                   int* iscal) {
  extern __shared__ __align__(16) unsigned char uncoverSmem[];
  uint32_t* s_idx = reinterpret_cast<uint32_t*>(uncoverSmem);          // [UNCOVER_CAP]
  int16_t* s_back = reinterpret_cast<int16_t*>(s_idx + UNCOVER_CAP);   // [UNCOVER_CAP][9]
  uint8_t* s_st = reinterpret_cast<uint8_t*>(s_back + 9 * UNCOVER_CAP);  // [UNCOVER_CAP]
  int n = min(iscal[IS_NUNCOVER], UNCOVER_CAP);
  // the count is consumed: zero it for the next step's collection
  __syncthreads();
  if (threadIdx.x == 0) iscal[IS_NUNCOVER] = 0;
  if (n == 0) return;
  // the team: one thread per candidate (whole warps, at most the block)
  // resolves the types, synchronising on named barrier 1, so that a handful
  // of candidates costs a handful of warps' barriers, not 32; the other
  // threads wait at the block barrier before the initialisation
  const int T = min((int)blockDim.x, (n + 31) & ~31);
  __shared__ int s_n;
  // node::initialize(initDensity, initVelocity or 0, mass, visc, lbF): the
  // equilibria depend only on the direction and on whether the node becomes
  // fluid (initial velocity) or interface (none), so the 2 x 19 values are
  // formed once, by the block's last threads while the others resolve
  __shared__ double s_feq[2][Q];
  const double rho0 = k.initDensity;
  {
    const int q = (int)blockDim.x - 1 - (int)threadIdx.x;
    if (q < 2 * Q) {
      const int c = q / Q, j = q - c * Q;
      const double vx = c == 0 ? k.initVel[0] : 0.0, vy = c == 0 ? k.initVel[1] : 0.0,
                   vz = c == 0 ? k.initVel[2] : 0.0;
      const double ux = k.lbF[0] / 2.0 / rho0 + vx, uy = k.lbF[1] / 2.0 / rho0 + vy,
                   uz = k.lbF[2] / 2.0 / rho0 + vz;
      const double usq = ux * ux + uy * uy + uz * uz;
      s_feq[c][j] = feqj(j, rho0, ux, uy, uz, usq);
    }
  }
  if (n <= 64 && k.nObj == 1) {
    // up to 64 candidates of one impactor: warp 0 alone, one or two
    // candidates per lane, in registers (no duplicates: one object box)
    if (threadIdx.x < 32) {
      if (n <= 32) uncoverResolveWarp<1>(k, mask, list, n, s_idx, s_st, &s_n);
      else uncoverResolveWarp<2>(k, mask, list, n, s_idx, s_st, &s_n);
    }
  } else if ((int)threadIdx.x < T) {
  int p2 = 1;
  while (p2 < n) p2 <<= 1;
  for (int i = threadIdx.x; i < p2; i += T) s_idx[i] = i < n ? list[i] : 0xffffffffu;
  teamSync(T);
  // bitonic sort ascending
  for (int size = 2; size <= p2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < p2; i += T) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const uint32_t a = s_idx[i], b = s_idx[j];
          if ((a > b) == up) {
            s_idx[i] = b;
            s_idx[j] = a;
          }
        }
      }
      teamSync(T);
    }
  // the same node can appear once per object box: drop duplicates
  if (k.nObj > 1) {
    if (threadIdx.x == 0) {
      int w = 0;
      for (int i = 0; i < n; ++i)
        if (i == 0 || s_idx[i] != s_idx[i - 1]) s_idx[w++] = s_idx[i];
      s_n = w;
    }
    teamSync(T);
    n = s_n;
  }
  auto find = [&](uint32_t lk) -> int {  // binary search among the candidates
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
      const int mid = (lo + hi) >> 1;
      const uint32_t v = s_idx[mid];
      if (v == lk) return mid;
      if (v < lk) lo = mid + 1;
      else hi = mid - 1;
    }
    return -1;
  };
  // One pass over each candidate's links (within the lattice: an impactor
  // that reaches the outer layer turns wall nodes into impactor nodes):
  // - a non-candidate neighbour gives a fixed type: s_st bit 4 for a fluid,
  //   bit 5 for a gas neighbour;
  // - a lower-index candidate is recorded in s_back;
  // - a higher-index candidate reads as an impactor node and gives nothing.
  // s_st bits 0-3 hold the candidate's state, 12 while unresolved.
  for (int i = threadIdx.x; i < n; i += T) {
    const uint32_t x = s_idx[i];
    int ix, iy, iz;
    coords(k, (long long)x, ix, iy, iz);
    // the neighbours' types, all loads issued before any is used
    uint8_t tls[Q];
#pragma unroll
    for (int j = 1; j < Q; ++j) {
      const int tx = ix + CX(j), ty = iy + CY(j), tz = iz + CZ(j);
      const bool in = tx >= 0 && tx < k.X && ty >= 0 && ty < k.Y && tz >= 0 && tz < k.Z;
      tls[j] = in ? (uint8_t)(mask[x + (uint32_t)nbrOffset(k, j)] & TYPE_MASK) : (uint8_t)0xFF;
    }
    uint8_t fix = 0;
    int nb = 0;
#pragma unroll
    for (int j = 1; j < Q; ++j) {
      if (tls[j] == 0xFF) continue;
      const uint32_t lk = x + (uint32_t)nbrOffset(k, j);
      const int mid = find(lk);
      if (mid < 0) {
        const int tl = tls[j];
        fix |= (uint8_t)((tl == 0 ? 0x10 : 0) | (tl == 2 ? 0x20 : 0));
      } else if (mid < i && nb < 9) {
        s_back[9 * i + nb++] = (int16_t)mid;
      }
    }
    for (int b = nb; b < 9; ++b) s_back[9 * i + b] = -1;
    if (onOuterLayer(k, ix, iy, iz)) fix |= 0x40;
    s_st[i] = (uint8_t)(12 | fix);
  }
  teamSync(T);
  // the new state of candidate i from the states of its lower-index
  // candidate neighbours and its fixed neighbour bits
  auto resolve = [&](int i) -> uint8_t {
    const uint8_t me = s_st[i];
    bool fluidNb = (me & 0x10) != 0, gasNb = (me & 0x20) != 0;
#pragma unroll
    for (int b = 0; b < 9; ++b) {
      const int m = s_back[9 * i + b];
      if (m < 0) break;
      const int tl = s_st[m] & 0x0F;
      fluidNb |= tl == 0;
      gasNb |= tl == 2;
    }
    return (uint8_t)((me & 0x70) | ((!fluidNb || (me & 0x40)) ? 2 : gasNb ? 3 : 0));
  };
  if (n <= UNCOVER_SERIAL) {
    // few candidates: one thread in ascending order, the reference's own
    // serial order (each sees the lower-index ones already resolved)
    if (threadIdx.x == 0)
      for (int i = 0; i < n; ++i) s_st[i] = resolve(i);
  } else {
    // many: fixed-point iteration, every candidate at once; the lower-index
    // dependencies form chains, so it settles within n + 1 rounds
    for (int iter = 0; iter <= n; ++iter) {
      int changed = 0;
      uint8_t nst[UNCOVER_CAP / 1024];
#pragma unroll
      for (int q = 0; q < UNCOVER_CAP / 1024; ++q) {
        const int i = threadIdx.x + q * T;
        if (i < n) nst[q] = resolve(i);
      }
      teamSync(T);
#pragma unroll
      for (int q = 0; q < UNCOVER_CAP / 1024; ++q) {
        const int i = threadIdx.x + q * T;
        if (i < n && s_st[i] != nst[q]) {
          s_st[i] = nst[q];
          changed = 1;
        }
      }
      if (!teamOr(T, changed)) break;
    }
  }
  teamSync(T);
  if (threadIdx.x == 0) s_n = n;
  }  // the team
  // the new nodes' initialisation by the whole block, one (node, direction)
  // per thread: the equilibria are FP64, and a thread per node would form
  // nineteen of them one after the other
  __syncthreads();
  n = s_n;
  for (int q = threadIdx.x; q < n * Q; q += blockDim.x) {
    const int i = q / Q, j = q - i * Q;
    const long long x = s_idx[i];
    const int st = s_st[i] & 0x0F;
    if (j == 0) {
      const uint8_t m = mask[x];
      mask[x] = (uint8_t)((m & ~TYPE_MASK) | st);
      if (st != 2) markActive(k, x);
      if (st == 2) mass[x] = 0.0;
    }
    if (st == 2) continue;
    fset(k, f, j, x, s_feq[st == 0 ? 0 : 1][j]);
    if (j == 0) {
      mass[x] = st == 0 ? rho0 : 0.5 * rho0;
      if (k.mixed && st == 0) nF[x] = (float)rho0;
      if (k.visc) k.visc[x] = k.initVisc;
    }
  }
}

// Voxelisation of the impactors (updateObjectBoundaries, src/LB.cpp:806-840).
__device__ __forceinline__ void voxelizeObjectsBody(const Consts& k, uint8_t* mask,
                                                    uint32_t* solid, uint8_t* objIdx,
                                                    double* mass, double* obj) {
  __shared__ SphereL sph[MAX_OBJ];
  loadSpheres(k, obj, OB_X0, sph);
  __syncthreads();
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {-1, -1, -1};
  for (int o = 0; o < k.nObj; ++o)
    for (int a = 0; a < 3; ++a) {
      lo[a] = min(lo[a], sph[o].lo[a]);
      hi[a] = max(hi[a], sph[o].hi[a]);
    }
  if (hi[0] < 0) return;
  // a box within the lattice: its volume fits 32 bits, as node indices do
  // (an empty box visits nothing)
  const bool boxOk = hi[0] >= lo[0] && hi[1] >= lo[1] && hi[2] >= lo[2];
  const unsigned nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
  const unsigned vol = boxOk ? nx * ny * nz : 0u;
  const unsigned stride = gridDim.x * blockDim.x;
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  BoxWalk bw(i, stride, nx, ny);
  for (; i < vol; i += stride, bw.next(nx, ny)) {
    const int ix = lo[0] + (int)bw.bx, iy = lo[1] + (int)bw.by, iz = lo[2] + (int)bw.bz;
    const long long x = ix + iy * k.sy + iz * k.sz;
    int last = -1;
    for (int o = 0; o < k.nObj; ++o)
      if (insideBox(sph[o].t, ix, iy, iz)) last = o;
    // the box reaches one node past the sphere, so it holds every neighbour
    // of a node turned into an impactor node: drop their neighbour cache
    const uint8_t m0 = mask[x];
    if (last < 0) {
      if (m0 & BULK) mask[x] = (uint8_t)(m0 & ~BULK);
      continue;
    }
    mask[x] = (uint8_t)((m0 & ~(TYPE_MASK | BULK | OSTALE)) | 12);
    solid[x] = (uint32_t)obj[last * OB_STRIDE + OB_INDEX];
    objIdx[x] = (uint8_t)last;
    mass[x] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x < (unsigned)k.nObj)
    for (int c = 0; c < 3; ++c)
      obj[threadIdx.x * OB_STRIDE + OB_X0PREV + c] = obj[threadIdx.x * OB_STRIDE + OB_X0 + c];
}

// updateIndices, step 1: every particle claims the nodes of the last active
// list inside it; the highest particle index wins (src/LB.cpp:695-710).
__device__ __forceinline__ void flagClaimBody(const Consts& k, const uint8_t* mask,
                                              uint32_t* claim, const double* px0,
                                              const double* pr, const int* iscal,
                                              unsigned long long* uscal) {
  if (!iscal[IS_NEWNBR]) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) uscal[US_FIRSTFLAG] = ~0ull;
  const int P = k.nPart;
  const int warpsPerBlock = blockDim.x >> 5;
  const int lane = threadIdx.x & 31;
  for (int p = blockIdx.x * warpsPerBlock + (threadIdx.x >> 5); p < P;
       p += gridDim.x * warpsPerBlock) {
    const double cx = px0[p] / k.uLength, cy = px0[P + p] / k.uLength,
                 cz = px0[2 * P + p] / k.uLength, r = pr[p] / k.uLength;
    int lo[3], hi[3];
    sphereBox(k, cx, cy, cz, r, lo, hi);
    const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    if (nx <= 0 || ny <= 0 || nz <= 0) continue;
    const int vol = nx * ny * nz;
    const SphereBoxTest st = sphereBoxTest(cx, cy, cz, r, lo);
    // lane l visits box nodes l, l + 32, ...: its box coordinates advance by
    // the decomposition of 32 with carries (no division per node), and nodes
    // clearly outside the sphere are dropped before their mask is read
    int bx = lane % nx, by = (lane / nx) % ny, bz = lane / (nx * ny);
    const int sx = 32 % nx, sy = (32 / nx) % ny, sz = 32 / (nx * ny);
    for (int i = lane; i < vol; i += 32) {
      const int ix = lo[0] + bx, iy = lo[1] + by, iz = lo[2] + bz;
      bx += sx;
      by += sy;
      bz += sz;
      if (bx >= nx) {
        bx -= nx;
        ++by;
      }
      if (by >= ny) {
        by -= ny;
        ++bz;
      }
      const float dx = (float)(ix - lo[0]) - st.fx, dy = (float)(iy - lo[1]) - st.fy,
                  dz = (float)(iz - lo[2]) - st.fz;
      if (dx * dx + dy * dy + dz * dz > st.r2out) continue;
      const long long x = ix + iy * k.sy + iz * k.sz;
      if (!(mask[x] & ABIT)) continue;
      if (insideBox(st, ix, iy, iz)) atomicMax(claim + x, (uint32_t)p + 1u);
    }
  }
}

// updateIndices, step 2: the flag reset of every node (solid index 0, walls
// included) and the new flags (src/LB.cpp:689-693).
__device__ __forceinline__ void flagApplyBody(const Consts& k, uint8_t* mask, uint32_t* solid,
                                              uint32_t* claim, int* iscal,
                                              unsigned long long* uscal) {
  if (!iscal[IS_NEWNBR]) return;
  // wall nodes are never claimed: from here on their solid index is 0
  if (blockIdx.x == 0 && threadIdx.x == 0) iscal[IS_WALLS_RESET] = 1;
  unsigned long long first = ~0ull;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < k.N;
       x += (long long)gridDim.x * blockDim.x) {
    const uint32_t c = claim[x];
    const uint8_t m = mask[x];
    const uint8_t nm = (uint8_t)(c ? (m | PFLAG) : (m & ~PFLAG));
    if (nm != m) mask[x] = nm;
    solid[x] = c ? c - 1u : 0u;
    if (c) {
      claim[x] = 0;
      if ((unsigned long long)x < first) first = (unsigned long long)x;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, first, o);
    first = v < first ? v : first;
  }
  if ((threadIdx.x & 31) == 0 && first != ~0ull) atomicMin(uscal + US_FIRSTFLAG, first);
}

// LB::findNewActive (one CTA): walk the flagged nodes in ascending order,
// un-flag those no longer inside their particle and stop at the first one
// that still is (the reference's loop-exiting break, src/LB.cpp:2001-2007).
__device__ __forceinline__ void findNewActiveBody(const Consts& k, uint8_t* mask,
                                                  uint32_t* solid, const double* px0,
                                                  const double* pr, int* iscal,
                                                  unsigned long long* uscal) {
  __shared__ unsigned long long s_min;
  if (threadIdx.x == 0) iscal[IS_NEWNBR] = 0;
  unsigned long long start = uscal[US_FIRSTFLAG];
  const int P = k.nPart;
  while (start < (unsigned long long)k.N) {
    if (threadIdx.x == 0) s_min = ~0ull;
    __syncthreads();
    const long long x = (long long)start + threadIdx.x;
    bool flagged = false, inside = false;
    if (x < k.N) {
      flagged = (mask[x] & PFLAG) != 0;
      if (flagged) {
        const uint32_t pid = solid[x];
        if (pid >= (uint32_t)P) {
          atomicOr(iscal + IS_ERROR, ERR_PARTICLE_INDEX);
        } else {
          int ix, iy, iz;
          coords(k, x, ix, iy, iz);
          // FP32 test with the centre and radius from FP32 products; within
          // a band around the surface that covers its error, the FP64 test
          // with the reference's quotients decides (the same answer)
          const float cx = (float)px0[pid] * k.invLengthF, cy = (float)px0[P + pid] * k.invLengthF,
                      cz = (float)px0[2 * P + pid] * k.invLengthF, rf = (float)pr[pid] * k.invLengthF;
          const float dx = (float)ix - cx, dy = (float)iy - cy, dz = (float)iz - cz;
          const float d2 = dx * dx + dy * dy + dz * dz, r2 = rf * rf;
          const float band = 8.0f * (rf + 1.0f) * k.posErrF + 1e-5f * r2 + 1e-5f;
          if (d2 < r2 - band) inside = true;
          else if (d2 > r2 + band) inside = false;
          else
            inside = insideSphere((double)ix, (double)iy, (double)iz, px0[pid] / k.uLength,
                                  px0[P + pid] / k.uLength, px0[2 * P + pid] / k.uLength,
                                  pr[pid] / k.uLength);
        }
        if (inside) atomicMin(&s_min, (unsigned long long)x);
      }
    }
    __syncthreads();
    const unsigned long long stop = s_min;
    if (flagged && (unsigned long long)x < stop) {
      mask[x] = (uint8_t)(mask[x] & ~PFLAG);
      solid[x] = 0;
    }
    __syncthreads();
    if (stop != ~0ull) {
      if (threadIdx.x == 0) uscal[US_FIRSTFLAG] = stop;
      return;
    }
    start += blockDim.x;
  }
  if (threadIdx.x == 0) uscal[US_FIRSTFLAG] = ~0ull;
}

// ---- initialisation (LB::latticeBolzmannInit) ------------------------------

// ---- entry points of the kernels above with their own parameter lists: one
// run (arguments by value) and many runs at once (blockIdx.z = run, record
// staged in shared memory) ----

#define JOB_PROLOGUE                                                  \
  __shared__ __align__(16) Consts sk;                                 \
  stageRecord(sk, jobs[blockIdx.z].k);                                \
  __syncthreads();                                                    \
  const CoupArgs& c = jobs[blockIdx.z].cp;

__global__ void lbPrepare(Consts k, double* pAcc, long long pAccLen, float* pAccF,
                          long long pAccFLen, double* obj, double* wallF, double* scal,
                          int* iscal, const double* px0, const double* px1, const double* pw1,
                          double* pkd, float* pkf) {
  lbPrepareBody(k, pAcc, pAccLen, pAccF, pAccFLen, obj, wallF, scal, iscal, px0, px1, pw1, pkd,
                pkf);
}
__global__ void lbPrepareBatch(const JobArgs* jobs) {
  JOB_PROLOGUE
  lbPrepareBody(sk, c.pAcc, c.pAccLen, c.pAccF, c.pAccFLen, c.obj, c.wallF, c.scal, c.iscal,
                c.px0, c.px1, c.pw1, c.pkd, c.pkf);
}

__global__ void lbFinalizeKernel(Consts k, double* pF, double* pM, double* pV, double* obj,
                                 double* wallF, double* scal, const int* iscal,
                                 const float* pAccF, double* pS, FsArgs fa, int redistribute) {
  lbFinalizeBody(k, pF, pM, pV, obj, wallF, scal, iscal, pAccF, pS, fa, redistribute);
}
__global__ void lbFinalizeKernelBatch(const JobArgs* jobs) {
  JOB_PROLOGUE
  lbFinalizeBody(sk, c.pF, c.pM, c.pV, c.obj, c.wallF, c.scal, c.iscal, c.pAccF, c.pS,
                 jobs[blockIdx.z].fs, c.redistribute);
}

__global__ void uncoverCollect(Consts k, const uint8_t* mask, const uint32_t* solid,
                               const double* obj, uint32_t* list, int* iscal) {
  uncoverCollectBody(k, mask, solid, obj, list, iscal);
}
__global__ void uncoverCollectBatch(const JobArgs* jobs) {
  JOB_PROLOGUE
  uncoverCollectBody(sk, c.mask, c.solid, c.obj, c.uncover, c.iscal);
}

__global__ void __launch_bounds__(1024) uncoverResolve(Consts k, uint8_t* mask, void* f,
                                                       double* mass, float* nF, uint32_t* list,
                                                       int* iscal) {
  uncoverResolveBody(k, mask, f, mass, nF, list, iscal);
}
__global__ void __launch_bounds__(1024) uncoverResolveBatch(const JobArgs* jobs) {
  JOB_PROLOGUE
  uncoverResolveBody(sk, c.mask, c.fcur, c.mass, c.nF, c.uncover, c.iscal);
}

__global__ void voxelizeObjects(Consts k, uint8_t* mask, uint32_t* solid, uint8_t* objIdx,
                                double* mass, double* obj) {
  voxelizeObjectsBody(k, mask, solid, objIdx, mass, obj);
}
__global__ void voxelizeObjectsBatch(const JobArgs* jobs) {
  JOB_PROLOGUE
  voxelizeObjectsBody(sk, c.mask, c.solid, c.objIdx, c.mass, c.obj);
}

__global__ void flagClaim(Consts k, const uint8_t* mask, uint32_t* claim, const double* px0,
                          const double* pr, const int* iscal, unsigned long long* uscal) {
  flagClaimBody(k, mask, claim, px0, pr, iscal, uscal);
}
__global__ void flagClaimBatch(const JobArgs* jobs) {
  JOB_PROLOGUE
  flagClaimBody(sk, c.mask, c.claim, c.px0, c.pr, c.iscal, c.uscal);
}

__global__ void flagApply(Consts k, uint8_t* mask, uint32_t* solid, uint32_t* claim,
                          int* iscal, unsigned long long* uscal) {
  flagApplyBody(k, mask, solid, claim, iscal, uscal);
}
__global__ void flagApplyBatch(const JobArgs* jobs) {
  JOB_PROLOGUE
  flagApplyBody(sk, c.mask, c.solid, c.claim, c.iscal, c.uscal);
}

__global__ void __launch_bounds__(1024) findNewActiveKernel(Consts k, uint8_t* mask,
                                                            uint32_t* solid, const double* px0,
                                                            const double* pr, int* iscal,
                                                            unsigned long long* uscal) {
  findNewActiveBody(k, mask, solid, px0, pr, iscal, uscal);
}
__global__ void __launch_bounds__(1024) findNewActiveKernelBatch(const JobArgs* jobs) {
  JOB_PROLOGUE
  findNewActiveBody(sk, c.mask, c.solid, c.px0, c.pr, c.iscal, c.uscal);
}

// initializeLatticeBoundaries, initializeWallBoundaries,
// initializeObjectBoundaries and initializeInterface (src/LB.cpp:538-795, 974-992)
__global__ void initTypes(Consts k, uint8_t* mask, uint32_t* solid, uint8_t* objIdx,
                          const int* boundary, const DeviceWall* walls, const int* wallType,
                          const double* obj, double fluidHeightLattice, int freeSurface) {
  // the quotients the reference forms at every node, formed once per block
  // (the same operands give the same double)
  __shared__ double wp[MAX_WALL][3], wn[MAX_WALL][3], oc[MAX_OBJ][4];
  __shared__ int wt[MAX_WALL];
  __shared__ uint32_t oidx[MAX_OBJ];
  if (threadIdx.x < (unsigned)k.nWall) {
    const DeviceWall& W = walls[threadIdx.x];
    for (int c = 0; c < 3; ++c) {
      wp[threadIdx.x][c] = W.p[c] / k.uLength;
      wn[threadIdx.x][c] = W.n[c];
    }
    wt[threadIdx.x] = wallType[threadIdx.x];
  }
  if (threadIdx.x < (unsigned)k.nObj) {
    const double* ob = obj + threadIdx.x * OB_STRIDE;
    for (int c = 0; c < 3; ++c) oc[threadIdx.x][c] = ob[OB_X0 + c] / k.uLength;
    oc[threadIdx.x][3] = ob[OB_R] / k.uLength;
    oidx[threadIdx.x] = (uint32_t)ob[OB_INDEX];
  }
  __syncthreads();
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < k.N;
       x += (long long)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    coords(k, x, ix, iy, iz);
    int t = 0;
    uint32_t so = 0;
    if (ix == 0) t = boundary[0];
    else if (ix == k.X - 1) t = boundary[1];
    else if (iy == 0) t = boundary[2];
    else if (iy == k.Y - 1) t = boundary[3];
    else if (iz == 0) t = boundary[4];
    else if (iz == k.Z - 1) t = boundary[5];
    const double p[3] = {(double)ix, (double)iy, (double)iz};
    for (int w = 0; w < k.nWall; ++w) {
      const double d = wn[w][0] * (p[0] - wp[w][0]) + wn[w][1] * (p[1] - wp[w][1]) +
                       wn[w][2] * (p[2] - wp[w][2]);
      if (d < 0.0) {
        so = (uint32_t)w;
        t = wt[w];
      }
    }
    uint8_t oi = 0;
    for (int o = 0; o < k.nObj; ++o) {
      if (insideSphereFast(p[0], p[1], p[2], oc[o][0], oc[o][1], oc[o][2], oc[o][3])) {
        so = oidx[o];
        t = 12;
        oi = (uint8_t)o;
      }
    }
    if (freeSurface && (double)(unsigned)iy > fluidHeightLattice && t == 0) t = 2;
    mask[x] = (uint8_t)t;
    solid[x] = so;
    objIdx[x] = oi;
  }
}

// initializeVariables (src/LB.cpp:1042-1096): fluid nodes next to gas become
// interface nodes; active nodes start at equilibrium. Typing in place is safe:
// a fluid->interface change never alters any node's gas neighbourhood. Also
// the first cleanLists (active-list bit).
__global__ void initFields(Consts k, uint8_t* mask, void* f, double* mass, float* nF,
                           double fluidHeightLattice, int freeSurface) {
  // every active node starts at the same equilibrium
  const double rho0 = k.initDensity;
  const double ux = k.lbF[0] / 2.0 / rho0 + k.initVel[0];
  const double uy = k.lbF[1] / 2.0 / rho0 + k.initVel[1];
  const double uz = k.lbF[2] / 2.0 / rho0 + k.initVel[2];
  const double usq = ux * ux + uy * uy + uz * uz;
  double feq[Q];
#pragma unroll
  for (int j = 0; j < Q; ++j) feq[j] = feqj(j, rho0, ux, uy, uz, usq);
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < k.N;
       x += (long long)gridDim.x * blockDim.x) {
    int t = mask[x] & TYPE_MASK;
    if (t == 0 && freeSurface) {
      // gas is only above the fill height (initTypes): a node whose upper
      // neighbours are below it has no gas neighbour
      const int iy = (int)((x / k.sy) % k.Y);
      if ((double)(unsigned)(iy + 1) > fluidHeightLattice)
        for (int j = 1; j < Q; ++j)
          if ((mask[x + nbrOffset(k, j)] & TYPE_MASK) == 2) {
            t = 3;
            break;
          }
    }
    double ms = 0.0;
    if (t == 0 || t == 3) {
#pragma unroll
      for (int j = 0; j < Q; ++j) fset(k, f, j, x, feq[j]);
      ms = t == 0 ? rho0 : 0.5 * rho0;
      mask[x] = (uint8_t)((mask[x] & ~TYPE_MASK) | t | ABIT);
      if (k.mixed && t == 0) nF[x] = (float)rho0;
    }
    mass[x] = ms;
  }
}

// every element of v[0 .. n) set to value (the initial per-node viscosity)
__global__ void fillDouble(double* v, long long n, double value) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
       x += (long long)gridDim.x * blockDim.x)
    v[x] = value;
}

// ---- slip walls (LB::streaming, src/LB.cpp:1454-1523) -------------------------
//
// For a diagonal link j (j > 6) of an active node x into a slip wall, the
// reference sets f_opp(x) = S1 fs_s(c) + S2 fs_j(x) when exactly one of the
// two nodes x + c_slip1Check[j], x + c_slip2Check[j] is active: c is that
// node and s = slip1[j] or slip2[j] respectively; otherwise (and for j <= 6)
// plain bounce-back. The lattice step has already bounced every wall link
// back, so after it fs_j(x) sits in direction opp(j) of x and fs_s(c) in
// direction opp(s) of c: the link s of c leads into the other check node,
// which is the inactive one and, for walls on the box faces, a wall node.
// As c's own value may be corrected in the same pass, slipStash first
// writes every corrected value into the wall node's slot of direction
// opp(j) (x + c_j, a slot no step reads), and slipApply then copies it to x.
template <bool APPLY>
__device__ __forceinline__ void slipPass(const Consts& k, const uint8_t* mask, void* f) {
  const long long NP = k.NP;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < k.N;
       x += (long long)gridDim.x * blockDim.x) {
    if (!isActiveT(mask[x] & TYPE_MASK)) continue;
    int ix, iy, iz;
    coords(k, x, ix, iy, iz);
    const unsigned wallN = boxWallLinks(k, ix, iy, iz);
    if (!(wallN >> 7)) continue;  // no diagonal link into a wall
    for (int j = 7; j < Q; ++j) {
      if (!((wallN >> j) & 1u)) continue;
      long long c;
      int s;
      if (!slipPartner(k, mask, x, j, c, s)) continue;
      const long long own = (long long)OPPJ(j) * NP + x;
      const long long stash = (long long)OPPJ(j) * NP + x + nbrOffset(k, j);
      if (k.mixed) {
        float* g = (float*)f;
        if (APPLY) g[own] = g[stash];
        else g[stash] = k.slipS1f * g[(long long)OPPJ(s) * NP + c] + k.slipS2f * g[own];
      } else {
        double* g = (double*)f;
        if (APPLY) g[own] = g[stash];
        else g[stash] = k.slipS1 * g[(long long)OPPJ(s) * NP + c] + k.slipS2 * g[own];
      }
    }
  }
}
__global__ void slipStash(Consts k, const uint8_t* mask, void* f) { slipPass<false>(k, mask, f); }
__global__ void slipApply(Consts k, const uint8_t* mask, void* f) { slipPass<true>(k, mask, f); }

// ---- diagnostics --------------------------------------------------------------

__global__ void massSummaryKernel(Consts k, const uint8_t* mask, const double* mass,
                                  const float* nF, double* out, unsigned long long* cnt,
                                  int withParticles) {
  double s = 0.0;
  unsigned long long ni = 0, na = 0;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < k.N;
       x += (long long)gridDim.x * blockDim.x) {
    const uint8_t m = mask[x];
    const int t = m & TYPE_MASK;
    if (isActiveT(t)) {
      ++na;
      if (t == 3) ++ni;
      if (withParticles || !(m & PFLAG)) s += (k.mixed && t == 0) ? (double)nF[x] : mass[x];
    }
  }
  blockAddDouble(s, true, out);
  for (int o = 16; o > 0; o >>= 1) {
    ni += __shfl_xor_sync(0xffffffffu, ni, o);
    na += __shfl_xor_sync(0xffffffffu, na, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(cnt, ni);
    atomicAdd(cnt + 1, na);
  }
}

// Moments of the current populations, for state download.
__global__ void momentsKernel(Consts k, const uint8_t* mask, const void* f, double* n,
                              double* u) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < k.N;
       x += (long long)gridDim.x * blockDim.x) {
    if (!isActiveT(mask[x] & TYPE_MASK)) {
      n[x] = 0.0;
      u[x] = u[k.N + x] = u[2 * k.N + x] = 0.0;
      continue;
    }
    double s = 0.0, ux = 0.0, uy = 0.0, uz = 0.0;
    for (int j = 0; j < Q; ++j) {
      const double fj = fget(k, f, j, x);
      s += fj;
      ux += CX(j) * fj;
      uy += CY(j) * fj;
      uz += CZ(j) * fj;
    }
    n[x] = s;
    u[x] = ux / s;
    u[k.N + x] = uy / s;
    u[2 * k.N + x] = uz / s;
  }
}

// Populations and masses of the active nodes as doubles, for state download.
__global__ void exportLattice(Consts k, const uint8_t* mask, const void* f, const double* mass,
                              const float* nF, double* fOut, double* massOut) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < k.N;
       x += (long long)gridDim.x * blockDim.x) {
    const int t = mask[x] & TYPE_MASK;
    const bool act = isActiveT(t);
    for (int j = 0; j < Q; ++j) fOut[(long long)j * k.N + x] = act ? fget(k, f, j, x) : 0.0;
    massOut[x] = (k.mixed && t == 0 && k.freeSurface) ? (double)nF[x] : mass[x];
  }
}

// Particle and impactor positions, velocities and hydrodynamic forces, and
// the interface mass share of the last step, finite (a few KB per run): the
// run server's check after each slice. A diverged lattice reaches the
// spheres' forces and the interface sums within cycles, and diverged
// contacts the spheres' motion.
__global__ void motionFiniteCheck(const double* px0, const double* px1, const double* pFH,
                                  int n3, const double* obj, int nObj, const double* scal,
                                  int* iscal) {
  bool bad = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x)
    bad |= !isfinite(px0[i]) || !isfinite(px1[i]) || !isfinite(pFH[i]);
  if (blockIdx.x == 0 && (int)threadIdx.x < 3 * nObj) {
    const double* ob = obj + (threadIdx.x / 3) * OB_STRIDE;
    const int c = threadIdx.x % 3;
    bad |= !isfinite(ob[OB_X0 + c]) || !isfinite(ob[OB_X1 + c]) || !isfinite(ob[OB_FHYDRO + c]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) bad |= !isfinite(scal[SC_ADD_MASS]);
  if (bad) atomicOr(iscal + IS_ERROR, ERR_NONFINITE);
}

__global__ void nonfiniteCheck(Consts k, const uint8_t* mask, const void* f, int* iscal) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < k.N;
       x += (long long)gridDim.x * blockDim.x) {
    if (!isActiveT(mask[x] & TYPE_MASK)) continue;
    double s = 0.0;
    for (int j = 0; j < Q; ++j) s += fget(k, f, j, x);
    if (!isfinite(s)) atomicOr(iscal + IS_ERROR, ERR_NONFINITE);
  }
}

}  // namespace lbdem
