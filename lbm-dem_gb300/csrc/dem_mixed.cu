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

// Mixed-form pair geometry from the FP64 separation d = xa - xb and relative
// velocity u = va - vb; rad is the mean radius (2 rad the contact distance).
__device__ __forceinline__ PairGeom<float> pairGeomM(double rad, const double* d,
                                                     const double* u) {
  PairGeom<float> g;
  const float dx = (float)d[0], dy = (float)d[1], dz = (float)d[2];
  const float r2 = dx * dx + dy * dy + dz * dz;
  const float lim = (float)((2.0 + NEAR_GAP) * rad);
  if (r2 < lim * lim) {
    const double r12 = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    g.r12 = (float)r12;
    g.gap = (float)(r12 - 2.0 * rad);
    g.n[0] = (float)(d[0] / r12);
    g.n[1] = (float)(d[1] / r12);
    g.n[2] = (float)(d[2] / r12);
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
    return (float)sqrt(ox * ox + oy * oy + oz * oz);
  }
  return l;
}

__device__ __forceinline__ void add3f(float* a, const float* b) {
  a[0] += b[0];
  a[1] += b[1];
  a[2] += b[2];
}
__device__ __forceinline__ void sub3f(float* a, const float* b) {
  a[0] -= b[0];
  a[1] -= b[1];
  a[2] -= b[2];
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
    double d[3], u[3];
    for (int c = 0; c < 3; ++c) {
      d[c] = a.x0[c * P + i] - a.x0[c * P + j];
      u[c] = a.x1[c * P + i] - a.x1[c * P + j];
    }
    float wa[3], wb[3];
    load3f(a.w1, P, i, wa);
    load3f(a.w1, P, j, wb);
    const double raD = a.r[i], rbD = a.r[j];
    const float ra = (float)raD, rb = (float)rbD;
    const PairGeom<float> g = pairGeomM(0.5 * (raD + rbD), d, u);
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

// Gather, wall and impactor terms and integration, one thread per particle:
// the plain form's demGather with FP32 force sums.
LBDEM_KERNEL(__launch_bounds__(GATHER_THREADS), demGatherMixed, DemArgs, dem) {
  const int stepNo = a.iscal[IS_DEMSTEP];
  __shared__ double acc[GA_N];
  __shared__ DeviceWall sW[MAX_WALL];
  __shared__ float sWp[MAX_WALL][3], sWn[MAX_WALL][3];
  for (int t = threadIdx.x; t < GA_N; t += blockDim.x) acc[t] = 0.0;
  if (threadIdx.x < (unsigned)k.nWall) {
    const DeviceWall W = a.walls[threadIdx.x];
    sW[threadIdx.x] = W;
    for (int c = 0; c < 3; ++c) {
      sWp[threadIdx.x][c] = (float)W.p[c];
      sWn[threadIdx.x][c] = (float)W.n[c];
    }
  }
  __syncthreads();
  // reach of the wall forces beyond a particle's radius: the largest
  // lubrication range, plus a margin far above the FP32 error of the test
  const float wallReach =
      (float)tmax(k.lubCut, tmax(k.lubN, tmax(k.lubT, k.lubR))) + 0.01f;
  const int cur = a.iscal[IS_LISTCUR];
  const int* L = a.list[cur];
  const float* pbuf = reinterpret_cast<const float*>(a.pairbuf);
  const int P = k.nPart;
  const bool afterWait = stepNo >= k.objWaitTime;
  // particles in the cell list's order (from the last rebuild), so that a
  // warp holds neighbours in space and few of its lanes branch into the wall
  // terms; the particle index order where the direct-sum branch is in use
  const int* order = a.iscal[IS_DIRECT] ? nullptr : a.cellParts;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < P; t += gridDim.x * blockDim.x) {
    const int i = order ? order[t] : t;
    double xa[3], va[3];
    load3(a.x0, P, i, xa);
    load3(a.x1, P, i, va);
    double waD[3];
    load3(a.w1, P, i, waD);
    const float vaf[3] = {(float)va[0], (float)va[1], (float)va[2]};
    const float wa[3] = {(float)waD[0], (float)waD[1], (float)waD[2]};
    const double raD = a.r[i];
    const float ra = (float)raD;
    float FC[3] = {0, 0, 0}, MC[3] = {0, 0, 0}, FL[3] = {0, 0, 0}, ML[3] = {0, 0, 0},
          FR[3] = {0, 0, 0};
    float xiw[3], xio[3];
    load3f(a.xiw, P, i, xiw);
    load3f(a.xio, P, i, xio);
    // the terms of the totals, loaded up front
    double FH[3], MH[3], FG[3];
    load3(a.FHydro, P, i, FH);
    load3(a.MHydro, P, i, MH);
    load3(a.FGrav, P, i, FG);
    const double im = a.invm[i], iI = a.invI[i];
    const int* li = L + (long long)i * MAX_N;
    const int* pt = a.partner + (long long)i * MAX_N;
    const int cnt = li[0];
    // pairs: contact, electrostatics and (after the wait) lubrication, from
    // the slot of the pair's owner (the higher index)
#pragma unroll 4
    for (int s = 1; s <= cnt; ++s) {
      const int j = li[s];
      const bool own = j < i;
      const long long e = own ? (long long)i * MAX_N + s : (long long)j * MAX_N + pt[s];
      const float* pb = pbuf + e * PAIR_VALS;
      if (own) {
        add3f(FC, pb);
        add3f(FR, pb + 15);
      } else {
        sub3f(FC, pb);
        sub3f(FR, pb + 15);
      }
      MC[0] += ra * pb[3];
      MC[1] += ra * pb[4];
      MC[2] += ra * pb[5];
      if (afterWait && (a.pairflag[e] & 1)) {
        if (own) {
          add3f(FL, pb + 6);
          add3f(ML, pb + 9);
        } else {
          sub3f(FL, pb + 6);
          add3f(ML, pb + 12);
        }
      }
    }
    // walls a force can reach (FP32 distance test); the others give no
    // force and reset the wall spring, as the contact law does out of contact
    unsigned nearW = 0;
    {
      const float xf[3] = {(float)xa[0], (float)xa[1], (float)xa[2]};
      for (int w = 0; w < k.nWall; ++w) {
        float l2 = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float oc = (xf[c] - sWp[w][c]) * sWn[w][c] * sWn[w][c];
          l2 += oc * oc;
        }
        const float lim = ra + wallReach;
        if (l2 < lim * lim) nearW |= 1u << w;
      }
    }
    float df[3], dt[3];
    if (afterWait) {
      for (int w = 0; w < k.nWall; ++w) {
        if (!((nearW >> w) & 1u)) continue;
        float o[3];
        const float l = wallGeomM(sW[w], xa, raD, o);
        float F[3], Tq[3];
        if (wallLubOne(k, ra, vaf, wa, o[0], o[1], o[2], l, F, Tq)) {
          add3f(FL, F);
          add3f(ML, Tq);
          for (int c = 0; c < 3; ++c)
            if (F[c] != 0.0f) atomicAdd(&acc[GA_WALL + 6 * w + 3 + c], -(double)F[c]);
        }
      }
      for (int o = 0; o < k.nObj; ++o) {
        const double* ob = a.obj + o * OB_STRIDE;
        const double ro = ob[OB_R];
        double d[3], u[3];
        for (int c = 0; c < 3; ++c) {
          d[c] = xa[c] - ob[OB_X0 + c];
          u[c] = va[c] - ob[OB_X1 + c];
        }
        const PairGeom<float> g = pairGeomM(0.5 * (raD + ro), d, u);
        const float wo[3] = {(float)ob[OB_W1], (float)ob[OB_W1 + 1], (float)ob[OB_W1 + 2]};
        objContactOne(k, ra, (float)ro, g, wa, wo, xio, df, dt);
        add3f(FC, df);
        MC[0] += ra * dt[0];
        MC[1] += ra * dt[1];
        MC[2] += ra * dt[2];
        for (int c = 0; c < 3; ++c) {
          if (df[c] != 0.0f) atomicAdd(&acc[GA_OBJ + 12 * o + c], -(double)df[c]);
          if (dt[c] != 0.0f) atomicAdd(&acc[GA_OBJ + 12 * o + 3 + c], ro * (double)dt[c]);
        }
        float lo[9];
        if (pairLub(k, ra, (float)ro, g, wa, wo, lo)) {
          add3f(FL, lo);
          add3f(ML, lo + 3);
          for (int c = 0; c < 3; ++c) {
            if (lo[c] != 0.0f) atomicAdd(&acc[GA_OBJ + 12 * o + 6 + c], -(double)lo[c]);
            if (lo[6 + c] != 0.0f) atomicAdd(&acc[GA_OBJ + 12 * o + 9 + c], (double)lo[6 + c]);
          }
        }
      }
    } else {
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
          continue;
        }
        float o[3];
        const float l = wallGeomM(sW[w], xa, raD, o);
        wallContactOne(k, ra, vaf, wa, xiw, o[0], o[1], o[2], l, nst, df, dt);
        add3f(FC, df);
        MC[0] += ra * dt[0];
        MC[1] += ra * dt[1];
        MC[2] += ra * dt[2];
        for (int c = 0; c < 3; ++c)
          if (df[c] != 0.0f) atomicAdd(&acc[GA_WALL + 6 * w + c], -(double)df[c]);
      }
    }
    // totals and integration in FP64
    const double dtt = k.dt;
    for (int c = 0; c < 3; ++c) {
      const double FT = FH[c] + (double)FC[c] + (double)FL[c] + FG[c] + (double)FR[c];
      const double MT = MH[c] + (double)MC[c] + (double)ML[c];
      const double xn = xa[c] + (dtt * va[c] + dtt * dtt * FT * im);
      a.x0[c * P + i] = xn;
      if (c == 1) {  // particle::disp.y and x_i.y (src/DEM.cpp:2705, 2721-2724)
        a.dispY[i] = a.xinitY[i] - xn;
        if (stepNo == k.objWaitTime) a.xinitY[i] = xn;
      }
      a.x1[c * P + i] = va[c] + dtt * FT * im;
      a.w1[c * P + i] = waD[c] + dtt * MT * iI;
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
    const double v = acc[t];
    if (v == 0.0) continue;
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
