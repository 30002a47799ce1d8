// DEM force passes of the mixed form: the force laws of the plain form
// (dem_forces.cuh) evaluated in FP32, with FP64 kept for
// - the separation of every pair (differences of FP64 positions),
// - the gap and normal of near-contact pairs (gap below 0.05 of the mean
//   radius, contacts included), of near-wall particles and of particles
//   near an impactor,
// - the particle and impactor integration and the force totals it uses.
// The per-pair contributions are stored as floats in the pair buffer; the
// gather visits a particle's neighbour slots in slot order (any fixed order
// keeps the sums deterministic; the mixed form does not follow the plain
// form's order of the reference).
//
// Reference: DEM::evaluateForces (src/DEM.cpp:655-796) and the force
// functions it calls; integration src/DEM.cpp:2676-2765.
#include "dem_forces.cuh"

namespace lbdem {

namespace {

// gap below which a pair's geometry is taken in FP64, relative to the mean
// radius
constexpr double NEAR_GAP = 0.05;

__device__ __forceinline__ void load3f(const double* a, int P, int i, float* v) {
  v[0] = (float)a[i];
  v[1] = (float)a[P + i];
  v[2] = (float)a[2 * P + i];
}

// 1/sqrt(r2) for r2 > 0 in FP64 to about 1e-13 relative: the FP32 estimate
// refined by one Newton step (y (3 - r2 y^2) / 2), a handful of FP64
// operations where sqrt and a division take several times as many.
__device__ __forceinline__ double rsqrtNewton(double r2) {
  const double y = (double)rsqrtf((float)r2);
  return y * fma(-0.5 * r2, y * y, 1.5);
}

// Mixed-form pair geometry from the FP64 separation d = xa - xb and relative
// velocity u = va - vb; rad is the mean radius (2 rad the contact distance).
// Near contact the distance and gap are taken in FP64 (the gap is a small
// difference of large numbers), the unit normal in FP32.
__device__ __forceinline__ PairGeom<float> pairGeomM(double rad, const double* d,
                                                     const double* u) {
  PairGeom<float> g;
  const float dx = (float)d[0], dy = (float)d[1], dz = (float)d[2];
  const float r2 = dx * dx + dy * dy + dz * dz;
  const float lim = (float)((2.0 + NEAR_GAP) * rad);
  if (r2 < lim * lim) {
    const double r2d = fma(d[0], d[0], fma(d[1], d[1], d[2] * d[2]));
    const double y = rsqrtNewton(r2d);
    const double r12 = r2d * y;
    g.r12 = (float)r12;
    g.gap = (float)(r12 - 2.0 * rad);
    const float yf = (float)y;
    g.n[0] = dx * yf;
    g.n[1] = dy * yf;
    g.n[2] = dz * yf;
  } else {
    const float r12 = sqrtf(r2);
    g.r12 = r12;
    g.gap = r12 - (float)(2.0 * rad);
    const float inv = 1.0f / r12;
    g.n[0] = dx * inv;
    g.n[1] = dy * inv;
    g.n[2] = dz * inv;
  }
  g.u[0] = (float)u[0];
  g.u[1] = (float)u[1];
  g.u[2] = (float)u[2];
  return g;
}

// The same for a particle pair from the FP64 separation d and the FP32
// relative velocity u and radii; near contact the mean radius is taken from
// the FP64 radii of particles i and j.
__device__ __forceinline__ PairGeom<float> pairGeomMf(const DemArgs& a, int i, int j, float ra,
                                                      float rb, const double* d, const float* u) {
  PairGeom<float> g;
  const float dx = (float)d[0], dy = (float)d[1], dz = (float)d[2];
  const float r2 = dx * dx + dy * dy + dz * dz;
  const float lim = (float)(2.0 + NEAR_GAP) * (0.5f * (ra + rb));
  if (r2 < lim * lim) {
    const double rad = 0.5 * (a.r[i] + a.r[j]);
    const double r2d = fma(d[0], d[0], fma(d[1], d[1], d[2] * d[2]));
    const double y = rsqrtNewton(r2d);
    const double r12 = r2d * y;
    g.r12 = (float)r12;
    g.gap = (float)(r12 - 2.0 * rad);
    const float yf = (float)y;
    g.n[0] = dx * yf;
    g.n[1] = dy * yf;
    g.n[2] = dz * yf;
  } else {
    const float r12 = sqrtf(r2);
    g.r12 = r12;
    g.gap = r12 - (ra + rb);
    const float inv = 1.0f / r12;
    g.n[0] = dx * inv;
    g.n[1] = dy * inv;
    g.n[2] = dz * inv;
  }
  g.u[0] = u[0];
  g.u[1] = u[1];
  g.u[2] = u[2];
  return g;
}

// Offset of particle x from wall W along its normal, and its length: the
// differences from the wall point in FP64, the rest in FP32 except within
// NEAR_GAP radii of contact, where the offset is taken in FP64.
__device__ __forceinline__ float wallGeomM(const DeviceWall& W, const double* x, double r,
                                           float* o) {
  const double d0 = x[0] - W.p[0], d1 = x[1] - W.p[1], d2 = x[2] - W.p[2];
  const float n0 = (float)W.n[0], n1 = (float)W.n[1], n2 = (float)W.n[2];
  o[0] = (float)d0 * n0 * n0;
  o[1] = (float)d1 * n1 * n1;
  o[2] = (float)d2 * n2 * n2;
  const float l = sqrtf(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
  if (l < (float)((1.0 + NEAR_GAP) * r)) {
    const double ox = d0 * W.n[0] * W.n[0], oy = d1 * W.n[1] * W.n[1], oz = d2 * W.n[2] * W.n[2];
    o[0] = (float)ox;
    o[1] = (float)oy;
    o[2] = (float)oz;
    const double l2 = fma(ox, ox, fma(oy, oy, oz * oz));
    return l2 > 0.0 ? (float)(l2 * rsqrtNewton(l2)) : 0.0f;
  }
  return l;
}

__device__ __forceinline__ void add3f(float* a, const float* b) {
  a[0] += b[0];
  a[1] += b[1];
  a[2] += b[2];
}

}  // namespace

// Owner pass: every pair (n1 > n2) evaluated once from n1's slot, one thread
// per entry of the owner-pair list; contributions stored as floats.
LBDEM_KERNEL(, demPairsMixed, DemArgs, dem) {
  const bool lubOn = a.iscal[IS_DEMSTEP] >= k.objWaitTime;
  const int cur = a.iscal[IS_LISTCUR];
  const int* L = a.list[cur];
  double* XI = a.xi[cur];
  float* pb = reinterpret_cast<float*>(a.pairbuf);
  const int P = k.nPart;
  const int npairs = min(a.iscal[IS_NPAIRS], max(P, 1) * (MAX_N / 2));
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < npairs; e += gridDim.x * blockDim.x) {
    const int idx = a.pairList[e];
    const int i = idx / MAX_N, s = idx % MAX_N;
    const int j = L[idx];
    // separation in FP64 (near contact the gap is a small difference of
    // large numbers); velocities, angular velocities and radii from this
    // step's FP32 copies
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = a.x0[c * P + i] - a.x0[c * P + j];
    const float4 va4 = a.kinf[2 * i], vb4 = a.kinf[2 * j];
    const float4 wa4 = a.kinf[2 * i + 1], wb4 = a.kinf[2 * j + 1];
    const float wa[3] = {wa4.x, wa4.y, wa4.z}, wb[3] = {wb4.x, wb4.y, wb4.z};
    const float ra = va4.w, rb = vb4.w;
    const float uf[3] = {va4.x - vb4.x, va4.y - vb4.y, va4.z - vb4.z};
    const PairGeom<float> g = pairGeomMf(a, i, j, ra, rb, d, uf);
    float out[PAIR_VALS];
    uint8_t flag = 0;
    if (lubOn && pairLub(k, ra, rb, g, wa, wb, out + 6)) flag |= 1;
    double* xii = XI + (long long)i * 3 * MAX_N;
    float xi[3] = {(float)xii[s], (float)xii[MAX_N + s], (float)xii[2 * MAX_N + s]};
    pairContact(k, ra, rb, g, wa, wb, xi, out);
    xii[s] = xi[0];
    xii[MAX_N + s] = xi[1];
    xii[2 * MAX_N + s] = xi[2];
    pairRep(k, g, out + 15);
    float* o = pb + (long long)idx * PAIR_VALS;
#pragma unroll
    for (int c = 0; c < 6; ++c) o[c] = out[c];
    if (flag & 1)
#pragma unroll
      for (int c = 6; c < 15; ++c) o[c] = out[c];
#pragma unroll
    for (int c = 15; c < 18; ++c) o[c] = out[c];
    a.pairflag[idx] = flag;
  }
}

// Pair sums of the gather: GATHER_MIXED_LANES lanes of a warp per particle,
// lane l summing the slots l+1, l+1+LANES, ... of the particle's list (the
// slot loop is a chain of dependent loads: spreading it over lanes hides
// their latency); the lanes' sums are combined by a fixed shuffle tree and
// stored per particle for demGatherMixed. FP32 only.
LBDEM_KERNEL(__launch_bounds__(GATHER_MIXED_THREADS), demSlotSumsMixed, DemArgs, dem) {
  const int cur = a.iscal[IS_LISTCUR];
  const int* L = a.list[cur];
  const float* pbuf = reinterpret_cast<const float*>(a.pairbuf);
  const int P = k.nPart;
  const bool afterWait = a.iscal[IS_DEMSTEP] >= k.objWaitTime;
  constexpr int LANES = GATHER_MIXED_LANES;
  const int sub = threadIdx.x % LANES;
  // warp-uniform loop: each warp takes 32/LANES consecutive particles
  const int first = blockIdx.x * GATHER_MIXED_PARTS + (threadIdx.x / 32) * (32 / LANES);
  for (int base = first; base < P; base += gridDim.x * GATHER_MIXED_PARTS) {
    const int i = base + (threadIdx.x % 32) / LANES;
    const bool valid = i < P;
    // pairs: contact, electrostatics and (after the wait) lubrication, from
    // the slot of the pair's owner (the higher index); the contact torques
    // are summed unscaled and multiplied by the radius in the gather
    float S[15];  // FC, MC / radius, FL, ML, FR
#pragma unroll
    for (int c = 0; c < 15; ++c) S[c] = 0.0f;
    if (valid) {
      const int* li = L + (long long)i * MAX_N;
      const int* pt = a.partner + (long long)i * MAX_N;
      const int cnt = li[0];
#pragma unroll 2
      for (int s = 1 + sub; s <= cnt; s += LANES) {
        const int j = li[s];
        const bool own = j < i;
        const long long e = own ? (long long)i * MAX_N + s : (long long)j * MAX_N + pt[s];
        const float* pb = pbuf + e * PAIR_VALS;
        const float sg = own ? 1.0f : -1.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          S[c] = __fmaf_rn(sg, pb[c], S[c]);
          S[3 + c] += pb[3 + c];
          S[12 + c] = __fmaf_rn(sg, pb[15 + c], S[12 + c]);
        }
        if (afterWait && (a.pairflag[e] & 1)) {
          const float* ml = pb + (own ? 9 : 12);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            S[6 + c] = __fmaf_rn(sg, pb[6 + c], S[6 + c]);
            S[9 + c] += ml[c];
          }
        }
      }
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1)
#pragma unroll
      for (int c = 0; c < 15; ++c) S[c] += __shfl_xor_sync(0xffffffffu, S[c], o);
    // lane c of the particle's group stores sum c (and c + LANES)
    if (valid) {
      float* out = a.slotSum + (size_t)i * SLOT_SUM_STRIDE;
#pragma unroll
      for (int c = 0; c < 15; ++c)
        if (c % LANES == sub) out[c] = S[c];
    }
  }
}

// The warp's sum of v added to *slot (one slot per warp: no atomics, a fixed
// order). Every lane of the warp calls it.
__device__ __forceinline__ void warpAccum(float v, float* slot) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) *slot += v;
}

// Gather, wall and impactor terms and integration, one thread per particle
// (every lane of a warp in the FP64 integration): the plain form's demGather
// with FP32 force sums, the pair sums from demSlotSumsMixed. The impactor
// and wall reactions are summed per warp in FP32 (a shuffle tree per term
// that any lane of the warp has) and per block in warp order, then added to
// the FP64 totals once per block: shared FP64 atomics from every particle at
// a wall serialise on their address.
LBDEM_KERNEL(__launch_bounds__(GATHER_THREADS), demGatherMixed, DemArgs, dem) {
  constexpr int NW = GATHER_THREADS / 32;
  const int stepNo = a.iscal[IS_DEMSTEP];
  // Each warp keeps its own reaction sums and its own copy of the wall and
  // impactor data in shared memory, so no block barrier stands between the
  // start of the kernel and the particle loads.
  __shared__ float acc[NW][GA_N];
  __shared__ DeviceWall sW[NW][MAX_WALL];
  __shared__ float sWp[NW][MAX_WALL][3], sWn[NW][MAX_WALL][3];
  __shared__ double sOb[NW][MAX_OBJ][10];  // r, x0, x1, w1
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* wacc = acc[wid];
  for (int t = lane; t < GA_N; t += 32) wacc[t] = 0.0f;
  if (lane < k.nWall) {
    const DeviceWall W = a.walls[lane];
    sW[wid][lane] = W;
    for (int c = 0; c < 3; ++c) {
      sWp[wid][lane][c] = (float)W.p[c];
      sWn[wid][lane][c] = (float)W.n[c];
    }
  }
  for (int t = lane; t < 10 * k.nObj; t += 32) {
    const int o = t / 10, c = t - o * 10;
    sOb[wid][o][c] = a.obj[o * OB_STRIDE + (c == 0 ? OB_R : c < 4 ? OB_X0 + c - 1
                                           : c < 7 ? OB_X1 + c - 4 : OB_W1 + c - 7)];
  }
  __syncwarp();
  // reach of the wall and impactor forces beyond the contact distance: the
  // largest lubrication range, plus a margin far above the FP32 error of the
  // distance tests
  const float wallReach =
      (float)tmax(k.lubCut, tmax(k.lubN, tmax(k.lubT, k.lubR))) + 0.01f;
  const int P = k.nPart;
  const bool afterWait = stepNo >= k.objWaitTime;
  const unsigned FULLM = 0xffffffffu;
  // particles in the cell list's order (from the last rebuild), so that a
  // warp holds neighbours in space and few of its lanes branch into the wall
  // terms; the particle index order where the direct-sum branch is in use
  const int* order = a.iscal[IS_DIRECT] ? nullptr : a.cellParts;
  // warp-uniform loop (the reaction sums take every lane)
  for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < P;
       base += gridDim.x * blockDim.x) {
    const int t = base + (threadIdx.x & 31);
    const bool valid = t < P;
    const int i = valid ? (order ? order[t] : t) : 0;
    double xa[3], va[3], waD[3];
    load3(a.x0, P, i, xa);
    load3(a.x1, P, i, va);
    load3(a.w1, P, i, waD);
    float xiw[3], xio[3];
    load3f(a.xiw, P, i, xiw);
    load3f(a.xio, P, i, xio);
    // the terms of the totals, loaded up front
    double FH[3], MH[3], FG[3];
    load3(a.FHydro, P, i, FH);
    load3(a.MHydro, P, i, MH);
    load3(a.FGrav, P, i, FG);
    const double im = a.invm[i], iI = a.invI[i];
    const double raD = a.r[i];
    const float4* ss = reinterpret_cast<const float4*>(a.slotSum + (size_t)i * SLOT_SUM_STRIDE);
    const float4 s0 = ss[0], s1 = ss[1], s2 = ss[2], s3 = ss[3];
    const float vaf[3] = {(float)va[0], (float)va[1], (float)va[2]};
    const float wa[3] = {(float)waD[0], (float)waD[1], (float)waD[2]};
    const float ra = (float)raD;
    float FC[3] = {s0.x, s0.y, s0.z}, MC[3] = {ra * s0.w, ra * s1.x, ra * s1.y},
          FL[3] = {s1.z, s1.w, s2.x}, ML[3] = {s2.y, s2.z, s2.w},
          FR[3] = {s3.x, s3.y, s3.z};
    // walls a force can reach (FP32 distance test); the others give no
    // force and reset the wall spring, as the contact law does out of contact
    unsigned nearW = 0;
    const float xf[3] = {(float)xa[0], (float)xa[1], (float)xa[2]};
    if (valid) {
      for (int w = 0; w < k.nWall; ++w) {
        float l2 = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float oc = (xf[c] - sWp[wid][w][c]) * sWn[wid][w][c] * sWn[wid][w][c];
          l2 += oc * oc;
        }
        const float lim = ra + wallReach;
        if (l2 < lim * lim) nearW |= 1u << w;
      }
    }
    const unsigned warpNearW = __reduce_or_sync(FULLM, nearW);
    float df[3], dt[3];
    if (afterWait) {
      for (int w = 0; w < k.nWall; ++w) {
        if (!((warpNearW >> w) & 1u)) continue;  // uniform
        float F[3] = {0.0f, 0.0f, 0.0f};
        if ((nearW >> w) & 1u) {
          float o[3], Tq[3];
          const float l = wallGeomM(sW[wid][w], xa, raD, o);
          if (wallLubOne(k, ra, vaf, wa, o[0], o[1], o[2], l, F, Tq)) {
            add3f(FL, F);
            add3f(ML, Tq);
          } else {
            F[0] = F[1] = F[2] = 0.0f;
          }
        }
        for (int c = 0; c < 3; ++c) warpAccum(-F[c], &wacc[GA_WALL + 6 * w + 3 + c]);
      }
      for (int o = 0; o < k.nObj; ++o) {
        const double* ob = sOb[wid][o];
        const double ro = ob[0];
        float R[12] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        bool any = false;
        // an impactor beyond the particle's reach gives no force and resets
        // the particle's impactor spring, as the contact law does out of
        // contact (FP32 distance test)
        bool nearO = false;
        if (valid) {
          const float ex = xf[0] - (float)ob[1], ey = xf[1] - (float)ob[2],
                      ez = xf[2] - (float)ob[3];
          const float lim = ra + (float)ro + wallReach;
          nearO = ex * ex + ey * ey + ez * ez < lim * lim;
          if (!nearO) xio[0] = xio[1] = xio[2] = 0.0f;
        }
        if (!__any_sync(FULLM, nearO)) continue;  // uniform
        if (nearO) {
          double d[3], u[3];
          for (int c = 0; c < 3; ++c) {
            d[c] = xa[c] - ob[1 + c];
            u[c] = va[c] - ob[4 + c];
          }
          const PairGeom<float> g = pairGeomM(0.5 * (raD + ro), d, u);
          const float wo[3] = {(float)ob[7], (float)ob[8], (float)ob[9]};
          objContactOne(k, ra, (float)ro, g, wa, wo, xio, df, dt);
          add3f(FC, df);
          MC[0] += ra * dt[0];
          MC[1] += ra * dt[1];
          MC[2] += ra * dt[2];
          const float rof = (float)ro;
          for (int c = 0; c < 3; ++c) {
            R[c] = -df[c];
            R[3 + c] = rof * dt[c];
          }
          float lo[9];
          if (pairLub(k, ra, rof, g, wa, wo, lo)) {
            add3f(FL, lo);
            add3f(ML, lo + 3);
            for (int c = 0; c < 3; ++c) {
              R[6 + c] = -lo[c];
              R[9 + c] = lo[6 + c];
            }
          }
          for (int c = 0; c < 12; ++c) any |= R[c] != 0.0f;
        }
        if (__any_sync(FULLM, any))
          for (int c = 0; c < 12; ++c) warpAccum(R[c], &wacc[GA_OBJ + 12 * o + c]);
      }
    } else if (valid) {
      float nst[3] = {0.0f, 0.0f, 0.0f};
      const double ylid = xa[1] - (k.demSize[1] - 0.3);
      wallContactOne(k, ra, vaf, wa, xiw, 0.0f, (float)ylid, 0.0f, (float)fabs(ylid), nst, df,
                     dt);
      add3f(FC, df);
      MC[0] += ra * dt[0];
      MC[1] += ra * dt[1];
      MC[2] += ra * dt[2];
    }
    // walls
    {
      float nst[3] = {0.0f, 0.0f, 0.0f};
      for (int w = 0; w < k.nWall; ++w) {
        if (!((nearW >> w) & 1u)) {
          xiw[0] = xiw[1] = xiw[2] = 0.0f;
        }
        if (!((warpNearW >> w) & 1u)) continue;  // uniform
        float F[3] = {0.0f, 0.0f, 0.0f};
        if ((nearW >> w) & 1u) {
          float o[3];
          const float l = wallGeomM(sW[wid][w], xa, raD, o);
          wallContactOne(k, ra, vaf, wa, xiw, o[0], o[1], o[2], l, nst, df, dt);
          add3f(FC, df);
          MC[0] += ra * dt[0];
          MC[1] += ra * dt[1];
          MC[2] += ra * dt[2];
          F[0] = df[0];
          F[1] = df[1];
          F[2] = df[2];
        }
        for (int c = 0; c < 3; ++c) warpAccum(-F[c], &wacc[GA_WALL + 6 * w + c]);
      }
    }
    if (!valid) continue;
    // totals in FP32 (the precision of the force sums), integration in FP64:
    // v' = v + dt F/m, x' = x + dt v + dt^2 F/m = x + dt v', w' = w + dt M/I
    const double dtt = k.dt;
    const double dtm = dtt * im, dtI = dtt * iI;
    for (int c = 0; c < 3; ++c) {
      const float FTf = (float)FH[c] + FC[c] + FL[c] + (float)FG[c] + FR[c];
      const float MTf = (float)MH[c] + MC[c] + ML[c];
      const double FT = (double)FTf, MT = (double)MTf;
      const double vn = fma(dtm, FT, va[c]);
      const double xn = fma(dtt, vn, xa[c]);
      a.x0[c * P + i] = xn;
      if (c == 1) {  // particle::disp.y and x_i.y (src/DEM.cpp:2705, 2721-2724)
        a.dispY[i] = a.xinitY[i] - xn;
        if (stepNo == k.objWaitTime) a.xinitY[i] = xn;
      }
      a.x1[c * P + i] = vn;
      a.w1[c * P + i] = fma(dtI, MT, waD[c]);
      a.FContact[c * P + i] = FC[c];
      a.MContact[c * P + i] = MC[c];
      a.FLub[c * P + i] = FL[c];
      a.MLub[c * P + i] = ML[c];
      a.FRep[c * P + i] = FR[c];
      a.FTotal[c * P + i] = FT;
      a.MTotal[c * P + i] = MT;
      a.xiw[c * P + i] = xiw[c];
      a.xio[c * P + i] = xio[c];
      if (stepNo <= k.objWaitTime) a.FGrav[c * P + i] = 0.0;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < GA_N; t += blockDim.x) {
    float vf = 0.0f;
#pragma unroll
    for (int w = 0; w < NW; ++w) vf += acc[w][t];
    if (vf == 0.0f) continue;
    const double v = (double)vf;
    if (t < GA_WALL) {
      const int o = t / 12, c = t % 12;
      const int off = c < 3 ? OB_FCONTACT + c : c < 6 ? OB_MCONTACT + c - 3
                    : c < 9 ? OB_FLUB + c - 6 : OB_MLUB + c - 9;
      atomicAdd(a.obj + o * OB_STRIDE + off, v);
    } else {
      const int w = (t - GA_WALL) / 6, c = (t - GA_WALL) % 6;
      atomicAdd(a.wallF + w * 12 + (c < 3 ? 3 + c : 6 + c - 3), v);
    }
  }
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(a.iscal + IS_GATHER_DONE, 1) == (int)gridDim.x - 1;
    if (last) a.iscal[IS_GATHER_DONE] = 0;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    demObjectsTail(k, a);
  }
}

}  // namespace lbdem
