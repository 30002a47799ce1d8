// DEM kernels (FP64): neighbour list (cell list with the reference's exact
// list order and tangential-history carry-over), pair forces (contact with
// Coulomb friction, Nguyen-Ladd lubrication, exponential electrostatic
// repulsion), particle-wall and particle-impactor terms, and the explicit
// integrator.
//
// Reference: DEM::discreteElementStep src/DEM.cpp:359-401, evalMaxDisp
// :460-470, neighborList :473-652, evaluateForces :655-796, pair/wall/object
// force functions :912-1340, 1404-1791, 1946-2672, integration :2676-2765.
//
// Structure: the reference visits each pair once from the higher index n1
// (whose list slot holds the tangential spring) and adds to both particles.
// Here the owner pass (demPairs) evaluates each pair once per owner slot and
// stores the pair's contributions; the gather pass (demGather) assembles
// every particle's sums in the reference's order (owner slots in slot
// order, then the pairs it appears in as n2 ordered by (n1, slot)), then
// adds the wall and impactor terms and integrates.
#include <cfloat>
#include <climits>

#include "dem_forces.cuh"
#include "kernels_decl.h"

namespace lbdem {

__device__ __forceinline__ int s_int(double x) { return x >= 0 ? (int)x : (int)(x - 1.0); }
__device__ __forceinline__ int n_int(double x) { return x >= 0 ? (int)(x + 0.5) : (int)(x - 0.5); }
__device__ __forceinline__ double boxf(double a, double b) { return a - s_int(a / b) * b; }
__device__ __forceinline__ double n_image(double a, double b) { return a - n_int(a / b) * b; }
// n_image without the division where |a| <= b/4: there a/b rounds into
// [-0.25, 0.25], n_int gives 0 and the result is a itself
__device__ __forceinline__ double n_image_near(double a, double b) {
  return fabs(a) <= 0.25 * b ? a : n_image(a, b);
}
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }


// ---- evalMaxDisp and the rebuild trigger -----------------------------------

// DEM::evalMaxDisp and the rebuild trigger of DEM::discreteElementStep
// (src/DEM.cpp:460-470, 368-378): the maximum of |x1|^2 over the particles
// (exact in any order: atomicMax on the bit patterns of non-negative
// doubles), then the last block to finish decides on a rebuild.
__device__ __forceinline__ void demBeginBody(const Consts& k, const DemArgs& a, int forceRebuild);
__global__ void __launch_bounds__(256) demBegin(Consts k, DemArgs a, int forceRebuild) {
  demBeginBody(k, a, forceRebuild);
}
__global__ void __launch_bounds__(256) demBeginBatch(const JobArgs* jobs) {
  __shared__ __align__(16) Consts sk;
  __shared__ __align__(16) DemArgs sa;
  stageRecord(sk, jobs[blockIdx.z].k);
  stageRecord(sa, jobs[blockIdx.z].dem);
  __syncthreads();
  demBeginBody(sk, sa, 0);
}
__device__ __forceinline__ void demBeginBody(const Consts& k, const DemArgs& a, int forceRebuild) {
  __shared__ double red[8];
  __shared__ bool last;
  double m = 0.0;
  const int P = k.nPart;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    const double vx = a.x1[i], vy = a.x1[P + i], vz = a.x1[2 * P + i];
    const double n2 = vx * vx + vy * vy + vz * vz;
    if (n2 > m) m = n2;
    if (a.kinf) {  // mixed form: this step's FP32 kinematics for the pair pass
      a.kinf[2 * i] = make_float4((float)vx, (float)vy, (float)vz, (float)a.r[i]);
      a.kinf[2 * i + 1] =
          make_float4((float)a.w1[i], (float)a.w1[P + i], (float)a.w1[2 * P + i], 0.0f);
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mv = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      if (red[w] > mv) mv = red[w];
    if (mv > 0.0)
      atomicMax(a.uscal + US_MAXV2, (unsigned long long)__double_as_longlong(mv));
    __threadfence();
    last = atomicAdd(a.iscal + IS_BLOCKS_DONE, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  if (threadIdx.x == 0) {
    __threadfence();
    double mv = __longlong_as_double((long long)atomicExch(a.uscal + US_MAXV2, 0ull));
    a.iscal[IS_BLOCKS_DONE] = 0;
    if (!forceRebuild) a.iscal[IS_DEMSTEP] += 1;  // ++demTimeStep (src/DEM.cpp:364)
    bool rebuild = forceRebuild != 0;
    if (!forceRebuild) {
      mv = sqrt(mv);
      a.scal[SC_MAXDISP] += mv * k.dt;
      if (a.scal[SC_MAXDISP] > 0.05) {
        a.scal[SC_MAXDISP] = 0.0;
        rebuild = true;
      }
    }
    a.iscal[IS_REBUILD] = rebuild ? 1 : 0;
    if (rebuild) {
      a.iscal[IS_NEWNBR] = 1;
      a.iscal[IS_REBUILDS] += 1;
      a.iscal[IS_NPAIRS] = 0;
    }
  }
  // reset of the per-step impactor and wall accumulators
  if (threadIdx.x < (unsigned)k.nObj) {
    double* ob = a.obj + threadIdx.x * OB_STRIDE;
    for (int c = 0; c < 3; ++c)
      ob[OB_FCONTACT + c] = ob[OB_MCONTACT + c] = ob[OB_FLUB + c] = ob[OB_MLUB + c] = 0.0;
  }
  if (threadIdx.x < (unsigned)k.nWall)
    for (int c = 3; c < 12; ++c) a.wallF[threadIdx.x * 12 + c] = 0.0;
}

// ---- neighbour list ---------------------------------------------------------

LBDEM_KERNEL(, nbrCellAssign, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD] || a.iscal[IS_DIRECT]) return;
  const int nlx = a.iscal[IS_NL], nly = a.iscal[IS_NL + 1], nlz = a.iscal[IS_NL + 2];
  const int P = k.nPart;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const double x = a.x0[p], y = a.x0[P + p], z = a.x0[2 * P + p];
    const int lx = (int)(boxf(x / k.demSize[0], 1) * nlx);
    const int ly = (int)(boxf(y / k.demSize[1], 1) * nly);
    const int lz = (int)(boxf(z / k.demSize[2], 1) * nlz);
    if (!(isfinite(x) && isfinite(y) && isfinite(z)) || lx < 0 || lx >= nlx || ly < 0 ||
        ly >= nly || lz < 0 || lz >= nlz) {
      atomicOr(a.iscal + IS_ERROR, ERR_GRID);
      a.pcell[p] = -1;
      continue;
    }
    const int l = lx * nly * nlz + ly * nlz + lz;
    a.pcell[p] = l;
    a.posf[p] = make_float4((float)x, (float)y, (float)z, (float)a.r[p]);
    atomicAdd(a.cellCount + l, 1);
  }
}

// exclusive scan of the cell counts (one CTA) and the occupancy check
LBDEM_KERNEL(__launch_bounds__(1024), nbrCellScan, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD] || a.iscal[IS_DIRECT]) return;
  __shared__ int carry;
  __shared__ int wsum[32];
  const int ncell = a.iscal[IS_NL] * a.iscal[IS_NL + 1] * a.iscal[IS_NL + 2];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < ncell; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < ncell ? a.cellCount[i] : 0;
    if (v > MAX_N) atomicOr(a.iscal + IS_ERROR, ERR_CELL_OVERFLOW);
    int s = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, s, o);
      if ((threadIdx.x & 31) >= o) s += t;
    }
    if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      int ws = threadIdx.x < (blockDim.x >> 5) ? wsum[threadIdx.x] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, ws, o);
        if (threadIdx.x >= o) ws += t;
      }
      wsum[threadIdx.x] = ws;
    }
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int excl = carry + (w ? wsum[w - 1] : 0) + s - v;
    if (i < ncell) {
      a.cellStart[i] = excl;
      a.cellFill[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
}

LBDEM_KERNEL(, nbrCellScatter, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD] || a.iscal[IS_DIRECT]) return;
  const int P = k.nPart;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int l = a.pcell[p];
    if (l < 0) continue;
    const int slot = atomicAdd(a.cellFill + l, 1);
    a.cellParts[a.cellStart[l] + slot] = p;
  }
}

// particles of a cell in ascending index order (the reference fills cells in
// particle order, src/DEM.cpp:567-583); positions are 1-based
LBDEM_KERNEL(, nbrCellSort, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD] || a.iscal[IS_DIRECT]) return;
  const int ncell = a.iscal[IS_NL] * a.iscal[IS_NL + 1] * a.iscal[IS_NL + 2];
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < ncell; l += gridDim.x * blockDim.x) {
    const int s = a.cellStart[l], n = a.cellCount[l];
    int* v = a.cellParts + s;
    for (int i = 1; i < n; ++i) {
      const int x = v[i];
      int j = i - 1;
      while (j >= 0 && v[j] > x) {
        v[j + 1] = v[j];
        --j;
      }
      v[j + 1] = x;
    }
    for (int i = 0; i < n; ++i) a.ppos[v[i]] = i + 1;
    a.cellCount[l] = 0;  // ready for the next rebuild
  }
}

__device__ __forceinline__ bool nbrWithin(const Consts& k, const double* x0, const double* r,
                                          int P, int n1, int n2);
// nbrWithin with an FP32 pre-test on the positions of the last cell
// assignment: the FP32 squared distance is within about 1e-3 (lu^2) of the
// FP64 one for lattice-sized boxes, so a pair well inside or well outside
// the cut-off gets the FP64 answer without FP64 arithmetic. Near the cut-off,
// or where a periodic image could apply, the FP64 test decides.
__device__ __forceinline__ bool nbrWithinFast(const Consts& k, const DemArgs& a, int P, int n1,
                                              int n2) {
  const float4 p1 = a.posf[n1], p2 = a.posf[n2];
  const float dx = p1.x - p2.x, dy = p1.y - p2.y, dz = p1.z - p2.z;
  const float qx = 0.25f * (float)k.demSize[0], qy = 0.25f * (float)k.demSize[1],
              qz = 0.25f * (float)k.demSize[2];
  if (fabsf(dx) < 0.99f * qx && fabsf(dy) < 0.99f * qy && fabsf(dz) < 0.99f * qz) {
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float cut = p1.w + p2.w + 2.0f;
    const float c2 = cut * cut;
    const float band = c2 * 1e-5f + 1e-2f;
    if (d2 < c2 - band) return true;
    if (d2 > c2 + band) return false;
  }
  return nbrWithin(k, a.x0, a.r, P, n1, n2);
}
__device__ __forceinline__ bool nbrWithin(const Consts& k, const double* x0, const double* r,
                                          int P, int n1, int n2) {
  const double x12 = n_image_near(x0[n1] - x0[n2], k.demSize[0]);
  const double y12 = n_image_near(x0[P + n1] - x0[P + n2], k.demSize[1]);
  const double z12 = n_image_near(x0[2 * P + n1] - x0[2 * P + n2], k.demSize[2]);
  const double r12 = x12 * x12 + y12 * y12 + z12 * z12;
  const double cut = r[n1] + r[n2] + 2.0;
  return r12 <= cut * cut;
}

// New list of each particle: the events of the reference's cell sweep that
// involve it, sorted by (cell l1, neighbour-cell order, position of n1 in
// l1, position of n2 in l2) - the order in which the reference appends them.
// NBR_GROUP lanes share a particle: they split its 54 cell visits (27
// neighbour cells, as n1 and as n2), collect the events in shared memory,
// place each event by its rank among the keys (keys are unique), and copy
// the tangential history slot by slot.
constexpr int NBR_GROUP = 8;
constexpr int NBR_PER_BLOCK = 128 / NBR_GROUP;
LBDEM_KERNEL(__launch_bounds__(128), nbrBuildCells, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD] || a.iscal[IS_DIRECT]) return;
  __shared__ unsigned long long sKey[NBR_PER_BLOCK][MAX_N];
  __shared__ int sNb[NBR_PER_BLOCK][MAX_N];
  __shared__ int sSorted[NBR_PER_BLOCK][MAX_N];
  __shared__ int sOld[NBR_PER_BLOCK][MAX_N];
  __shared__ int sCnt[NBR_PER_BLOCK];
  const int cur = a.iscal[IS_LISTCUR];
  const int* oldList = a.list[cur];
  const double* oldXi = a.xi[cur];
  int* newList = a.list[1 - cur];
  double* newXi = a.xi[1 - cur];
  const int nlx = a.iscal[IS_NL], nly = a.iscal[IS_NL + 1], nlz = a.iscal[IS_NL + 2];
  const int P = k.nPart;
  const int g = threadIdx.x / NBR_GROUP, sub = threadIdx.x % NBR_GROUP;
  // the loop bound is uniform over the block (it holds __syncthreads)
  for (int base = blockIdx.x * NBR_PER_BLOCK; base < P; base += gridDim.x * NBR_PER_BLOCK) {
    const int p = base + g;
    const int cp = p < P ? a.pcell[p] : -1;
    const bool valid = cp >= 0;
    if (sub == 0) sCnt[g] = 0;
    __syncthreads();
    // a cell coordinate shifted by -1, 0 or +1 wrapped into [0, n): the
    // reference's (c + d + n) % n for |d| <= 1
    auto wrap = [](int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); };
    if (valid) {
      const int cx = cp / (nly * nlz), cy = (cp / nlz) % nly, cz = cp % nlz;
      const int posp = a.ppos[p];
      // the old list of p, for the history copy below
      for (int l = sub; l < MAX_N; l += NBR_GROUP) sOld[g][l] = oldList[(long long)p * MAX_N + l];
      for (int v = sub; v < 54; v += NBR_GROUP) {
        const int kk = v >> 1;
        const int dx = kk / 9 - 1, dy = (kk / 3) % 3 - 1, dz = kk % 3 - 1;
        if ((v & 1) == 0) {
          // p as n1: partner q < p in l2 = l1 + d
          const int l2 = wrap(cx + dx, nlx) * nly * nlz + wrap(cy + dy, nly) * nlz +
                         wrap(cz + dz, nlz);
          const int s0 = a.cellStart[l2], n = a.cellFill[l2];
          for (int t = 0; t < n; ++t) {
            const int q = a.cellParts[s0 + t];
            if (q >= p || !nbrWithinFast(k, a, P, p, q)) continue;
            const int e = atomicAdd(&sCnt[g], 1);
            if (e >= MAX_N - 1) break;
            sKey[g][e] = ((unsigned long long)cp << 22) | ((unsigned long long)kk << 12) |
                         ((unsigned long long)posp << 6) | (unsigned long long)(t + 1);
            sNb[g][e] = q;
          }
        } else {
          // p as n2: partner q > p in l1 = l2 - d
          const int l1 = wrap(cx - dx, nlx) * nly * nlz + wrap(cy - dy, nly) * nlz +
                         wrap(cz - dz, nlz);
          const int s0 = a.cellStart[l1], n = a.cellFill[l1];
          for (int t = 0; t < n; ++t) {
            const int q = a.cellParts[s0 + t];
            if (q <= p || !nbrWithinFast(k, a, P, q, p)) continue;
            const int e = atomicAdd(&sCnt[g], 1);
            if (e >= MAX_N - 1) break;
            sKey[g][e] = ((unsigned long long)l1 << 22) | ((unsigned long long)kk << 12) |
                         ((unsigned long long)(t + 1) << 6) | (unsigned long long)posp;
            sNb[g][e] = q;
          }
        }
      }
    }
    __syncthreads();
    int cnt = 0;
    if (valid) {
      cnt = sCnt[g];
      if (cnt > MAX_N - 1) {
        if (sub == 0) atomicOr(a.iscal + IS_ERROR, ERR_NBR_OVERFLOW);
        cnt = MAX_N - 1;
      }
      for (int e = sub; e < cnt; e += NBR_GROUP) {
        const unsigned long long key = sKey[g][e];
        int rank = 0;
        for (int f = 0; f < cnt; ++f) rank += sKey[g][f] < key ? 1 : 0;
        sSorted[g][rank] = sNb[g][e];
      }
    }
    __syncthreads();
    if (valid) {
      const int* ol = sOld[g];
      const double* ox = oldXi + (long long)p * 3 * MAX_N;
      int* nl = newList + (long long)p * MAX_N;
      double* nx = newXi + (long long)p * 3 * MAX_N;
      if (sub == 0) {
        nl[0] = cnt;
        for (int c = 0; c < 3; ++c) nx[c * MAX_N] = (double)cnt;
      }
      // tangential history: last match in the old list wins; unmatched
      // slots keep their old value (src/DEM.cpp:633-651)
      const int ocnt = ol[0];
      for (int s = 1 + sub; s < MAX_N; s += NBR_GROUP) {
        int src = s;
        if (s <= cnt) {
          const int q = sSorted[g][s - 1];
          nl[s] = q;
          for (int l = 1; l <= ocnt; ++l)
            if (ol[l] == q) src = l;
        }
        for (int c = 0; c < 3; ++c) nx[c * MAX_N + s] = ox[c * MAX_N + src];
      }
    }
    __syncthreads();
  }
}

// Direct-sum branch (src/DEM.cpp:515-554): lists in (n1, n2) order.
LBDEM_KERNEL(, nbrBuildDirect, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD] || !a.iscal[IS_DIRECT]) return;
  const int cur = a.iscal[IS_LISTCUR];
  int* newList = a.list[1 - cur];
  const int P = k.nPart;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    int* nl = newList + (long long)p * MAX_N;
    int cnt = 0;
    bool over = false;
    for (int q = 0; q < P; ++q) {
      if (q == p) continue;
      const bool in = q < p ? nbrWithin(k, a.x0, a.r, P, p, q) : nbrWithin(k, a.x0, a.r, P, q, p);
      if (!in) continue;
      if (cnt >= MAX_N - 1) { over = true; break; }
      nl[++cnt] = q;
    }
    nl[0] = cnt;
    if (over) atomicOr(a.iscal + IS_ERROR, ERR_NBR_OVERFLOW);
  }
}

// Direct-sum history: unmatched slots take the value the reference's
// cross-copy leaves there (the old spring of n2 at n2's new slot).
LBDEM_KERNEL(, nbrDirectHistory, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD] || !a.iscal[IS_DIRECT]) return;
  const int cur = a.iscal[IS_LISTCUR];
  const int* oldList = a.list[cur];
  const double* oldXi = a.xi[cur];
  const int* newList = a.list[1 - cur];
  double* newXi = a.xi[1 - cur];
  const int P = k.nPart;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int* ol = oldList + (long long)p * MAX_N;
    const int* nl = newList + (long long)p * MAX_N;
    double* nx = newXi + (long long)p * 3 * MAX_N;
    const int cnt = nl[0], ocnt = ol[0];
    for (int s = 1; s < MAX_N; ++s) {
      const double* src = oldXi + (long long)p * 3 * MAX_N + s;
      if (s <= cnt) {
        const int q = nl[s];
        int match = -1;
        for (int l = 1; l <= ocnt; ++l)
          if (ol[l] == q) match = l;
        if (match >= 0) {
          src = oldXi + (long long)p * 3 * MAX_N + match;
        } else if (q < p) {
          const int* ql = newList + (long long)q * MAX_N;
          int c2 = 1;
          for (int t = 1; t <= ql[0]; ++t)
            if (ql[t] < p) ++c2;
          src = oldXi + (long long)q * 3 * MAX_N + c2;
        }
      }
      for (int c = 0; c < 3; ++c) nx[c * MAX_N + s] = src[c * MAX_N];
    }
    for (int c = 0; c < 3; ++c) nx[c * MAX_N] = (double)cnt;
  }
}

// Partner slots and the gather order of every list.
// One warp per particle: the lanes find the partner slots, lane 0 orders
// the gather (owner slots in slot order, then the partner slots by (n1,
// slot in n1's list)).
LBDEM_KERNEL(, nbrPartners, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD]) return;
  const int cur = 1 - a.iscal[IS_LISTCUR];
  const int* L = a.list[cur];
  const int P = k.nPart;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int i = blockIdx.x * wpb + (int)(threadIdx.x >> 5); i < P; i += gridDim.x * wpb) {
    const int* li = L + (long long)i * MAX_N;
    int* pt = a.partner + (long long)i * MAX_N;
    int* go = a.gorder + (long long)i * MAX_N;
    const int cnt = li[0];
    // slot s with j = li[s] > i: the occ-th appearance of i in j's list,
    // occ = the appearances of j in i's slots before s
    for (int s = 1 + lane; s <= cnt; s += 32) {
      const int j = li[s];
      int found = 0;
      if (j > i) {
        int occ = 0;
        for (int t = 1; t < s; ++t)
          if (li[t] == j) ++occ;
        const int* lj = L + (long long)j * MAX_N;
        int seen = 0;
        for (int t = 1; t <= lj[0]; ++t)
          if (lj[t] == i) {
            if (seen == occ) {
              found = t;
              break;
            }
            ++seen;
          }
      }
      pt[s] = found;
    }
    __syncwarp();
    if (lane == 0) {
      int ng = 0;
      for (int s = 1; s <= cnt; ++s)
        if (li[s] < i) go[ng++] = s;
      const int nown = ng;
      for (int s = 1; s <= cnt; ++s)
        if (li[s] > i) go[ng++] = s;
      // partner part ordered by (n1, slot in n1's list)
      for (int u = nown + 1; u < ng; ++u) {
        const int s = go[u];
        const long long key = (long long)li[s] * 64 + pt[s];
        int v = u - 1;
        while (v >= nown && (long long)li[go[v]] * 64 + pt[go[v]] > key) {
          go[v + 1] = go[v];
          --v;
        }
        go[v + 1] = s;
      }
    }
    __syncwarp();
  }
}

// Owner slots of the new lists (slot s of particle i with list[i][s] < i),
// so that the pair pass runs one thread per pair. The order of the entries
// does not matter: every pair writes only its own slot's outputs.
LBDEM_KERNEL(, nbrPairList, DemArgs, dem) {
  if (!a.iscal[IS_REBUILD]) return;
  const int* L = a.list[1 - a.iscal[IS_LISTCUR]];
  const long long total = (long long)k.nPart * MAX_N;
  const int cap = max(k.nPart, 1) * (MAX_N / 2);
  // one counter increment per warp (all lanes run the same iterations)
  const int lane = threadIdx.x & 31;
  for (long long b0 = blockIdx.x * (long long)blockDim.x; b0 < total;
       b0 += (long long)gridDim.x * blockDim.x) {
    const long long idx = b0 + threadIdx.x;
    bool own = false;
    if (idx < total) {
      const int s = (int)(idx % MAX_N);
      const int i = (int)(idx / MAX_N);
      own = s != 0 && s <= L[(long long)i * MAX_N] && L[idx] < i;
    }
    const unsigned m = __ballot_sync(0xffffffffu, own);
    int first = 0;
    if (lane == 0 && m) first = atomicAdd(a.iscal + IS_NPAIRS, __popc(m));
    first = __shfl_sync(0xffffffffu, first, 0);
    if (own) {
      const int pos = first + __popc(m & ((1u << lane) - 1u));
      if (pos < cap) a.pairList[pos] = (int)idx;
      else atomicOr(a.iscal + IS_ERROR, ERR_NBR_OVERFLOW);
    }
  }
  // the last block to finish makes the new lists current
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(a.iscal + IS_PAIRLIST_DONE, 1) == (int)gridDim.x - 1) {
      a.iscal[IS_PAIRLIST_DONE] = 0;
      a.iscal[IS_LISTCUR] = 1 - a.iscal[IS_LISTCUR];
    }
  }
}

// ---- pair forces (owner pass) ------------------------------------------------


// Owner pass: every pair (n1 > n2) evaluated once from n1's slot, one
// thread per entry of the owner-pair list.
LBDEM_KERNEL(, demPairs, DemArgs, dem) {
  // lubrication only after objWaitTime (src/DEM.cpp:716-725)
  const bool lubOn = a.iscal[IS_DEMSTEP] >= k.objWaitTime;
  const int cur = a.iscal[IS_LISTCUR];
  const int* L = a.list[cur];
  double* XI = a.xi[cur];
  const int P = k.nPart;
  const int npairs = min(a.iscal[IS_NPAIRS], max(P, 1) * (MAX_N / 2));
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < npairs; e += gridDim.x * blockDim.x) {
    const int idx = a.pairList[e];
    const int i = idx / MAX_N, s = idx % MAX_N;
    const int j = L[idx];
    double* xii = XI + (long long)i * 3 * MAX_N;
    double xa[3], va[3], wa[3], xb[3], vb[3], wb[3];
    load3(a.x0, P, i, xa);
    load3(a.x1, P, i, va);
    load3(a.w1, P, i, wa);
    load3(a.x0, P, j, xb);
    load3(a.x1, P, j, vb);
    load3(a.w1, P, j, wb);
    const double ra = a.r[i], rb = a.r[j];
    const PairGeom<double> g = pairGeomD(0.5 * (ra + rb), xa, xb, va, vb);
    double* out = a.pairbuf + (long long)idx * PAIR_VALS;
    uint8_t flag = 0;
    if (lubOn && pairLub(k, ra, rb, g, wa, wb, out + 6)) flag |= 1;
    double xi[3] = {xii[s], xii[MAX_N + s], xii[2 * MAX_N + s]};
    pairContact(k, ra, rb, g, wa, wb, xi, out);
    xii[s] = xi[0];
    xii[MAX_N + s] = xi[1];
    xii[2 * MAX_N + s] = xi[2];
    pairRep(k, g, out + 15);
    a.pairflag[idx] = flag;
  }
}

// ---- gather, walls, impactor, integration ------------------------------------




LBDEM_KERNEL(__launch_bounds__(GATHER_THREADS), demGather, DemArgs, dem) {
  const int stepNo = a.iscal[IS_DEMSTEP];
  __shared__ double acc[GA_N];
  for (int t = threadIdx.x; t < GA_N; t += blockDim.x) acc[t] = 0.0;
  __syncthreads();
  const int cur = a.iscal[IS_LISTCUR];
  const int* L = a.list[cur];
  const int P = k.nPart;
  const bool afterWait = stepNo >= k.objWaitTime;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    double xa[3], va[3], wa[3];
    load3(a.x0, P, i, xa);
    load3(a.x1, P, i, va);
    load3(a.w1, P, i, wa);
    const double ra = a.r[i];
    double FC[3] = {0, 0, 0}, MC[3] = {0, 0, 0}, FL[3] = {0, 0, 0}, ML[3] = {0, 0, 0},
           FR[3] = {0, 0, 0};
    double xiw[3], xio[3];
    load3(a.xiw, P, i, xiw);
    load3(a.xio, P, i, xio);
    const int* li = L + (long long)i * MAX_N;
    const int* go = a.gorder + (long long)i * MAX_N;
    const int* pt = a.partner + (long long)i * MAX_N;
    const int cnt = li[0];
    double df[3], dt[3];
    // lubrication first in evaluateForces (pairs, walls), then the impactor
    if (afterWait) {
      for (int u = 0; u < cnt; ++u) {
        const int s = go[u];
        const int j = li[s];
        if (j < i) {
          if (a.pairflag[(long long)i * MAX_N + s] & 1) {
            const double* pb = a.pairbuf + ((long long)i * MAX_N + s) * PAIR_VALS;
            add3(FL, pb + 6);
            add3(ML, pb + 9);
          }
        } else {
          const long long js = (long long)j * MAX_N + pt[s];
          if (a.pairflag[js] & 1) {
            const double* pb = a.pairbuf + js * PAIR_VALS;
            sub3(FL, pb + 6);
            add3(ML, pb + 12);
          }
        }
      }
      for (int w = 0; w < k.nWall; ++w) {
        const DeviceWall& W = a.walls[w];
        const double x12 = (xa[0] - W.p[0]) * W.n[0] * W.n[0];
        const double y12 = (xa[1] - W.p[1]) * W.n[1] * W.n[1];
        const double z12 = (xa[2] - W.p[2]) * W.n[2] * W.n[2];
        const double r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
        double F[3], T[3];
        if (wallLubOne(k, ra, va, wa, x12, y12, z12, r12, F, T)) {
          add3(FL, F);
          add3(ML, T);
          for (int c = 0; c < 3; ++c)
            if (F[c] != 0.0) atomicAdd(&acc[GA_WALL + 6 * w + 3 + c], -F[c]);
        }
      }
      for (int o = 0; o < k.nObj; ++o) {
        const double* ob = a.obj + o * OB_STRIDE;
        const PairGeom<double> g =
            pairGeomD(0.5 * (ra + ob[OB_R]), xa, ob + OB_X0, va, ob + OB_X1);
        objContactOne(k, ra, ob[OB_R], g, wa, ob + OB_W1, xio, df, dt);
        add3(FC, df);
        MC[0] += ra * dt[0];
        MC[1] += ra * dt[1];
        MC[2] += ra * dt[2];
        // a zero addend leaves a sum unchanged: only contacts touch the sums
        for (int c = 0; c < 3; ++c) {
          if (df[c] != 0.0) atomicAdd(&acc[GA_OBJ + 12 * o + c], -df[c]);
          if (dt[c] != 0.0) atomicAdd(&acc[GA_OBJ + 12 * o + 3 + c], ob[OB_R] * dt[c]);
        }
      }
      for (int o = 0; o < k.nObj; ++o) {
        const double* ob = a.obj + o * OB_STRIDE;
        double lo[9];
        const PairGeom<double> g =
            pairGeomD(0.5 * (ra + ob[OB_R]), xa, ob + OB_X0, va, ob + OB_X1);
        if (pairLub(k, ra, ob[OB_R], g, wa, ob + OB_W1, lo)) {
          add3(FL, lo);
          add3(ML, lo + 3);
          for (int c = 0; c < 3; ++c) {
            if (lo[c] != 0.0) atomicAdd(&acc[GA_OBJ + 12 * o + 6 + c], -lo[c]);
            if (lo[6 + c] != 0.0) atomicAdd(&acc[GA_OBJ + 12 * o + 9 + c], lo[6 + c]);
          }
        }
      }
    } else {
      double nst[3] = {0.0, 0.0, 0.0};
      const double ylid = xa[1] - (k.demSize[1] - 0.3);
      wallContactOne(k, ra, va, wa, xiw, 0.0, ylid, 0.0, sqrt(ylid * ylid), nst, df, dt);
      add3(FC, df);
      MC[0] += ra * dt[0];
      MC[1] += ra * dt[1];
      MC[2] += ra * dt[2];
    }
    // pair contact and electrostatics in the reference's pair order
    for (int u = 0; u < cnt; ++u) {
      const int s = go[u];
      const int j = li[s];
      if (j < i) {
        const double* pb = a.pairbuf + ((long long)i * MAX_N + s) * PAIR_VALS;
        add3(FC, pb);
        MC[0] += ra * pb[3];
        MC[1] += ra * pb[4];
        MC[2] += ra * pb[5];
      } else {
        const double* pb = a.pairbuf + ((long long)j * MAX_N + pt[s]) * PAIR_VALS;
        sub3(FC, pb);
        MC[0] += ra * pb[3];
        MC[1] += ra * pb[4];
        MC[2] += ra * pb[5];
      }
    }
    for (int u = 0; u < cnt; ++u) {
      const int s = go[u];
      const int j = li[s];
      if (j < i) add3(FR, a.pairbuf + ((long long)i * MAX_N + s) * PAIR_VALS + 15);
      else sub3(FR, a.pairbuf + ((long long)j * MAX_N + pt[s]) * PAIR_VALS + 15);
    }
    // walls
    {
      double nst[3] = {0.0, 0.0, 0.0};
      for (int w = 0; w < k.nWall; ++w) {
        const DeviceWall& W = a.walls[w];
        const double x1w = (xa[0] - W.p[0]) * W.n[0] * W.n[0];
        const double y1w = (xa[1] - W.p[1]) * W.n[1] * W.n[1];
        const double z1w = (xa[2] - W.p[2]) * W.n[2] * W.n[2];
        const double r1w = sqrt(x1w * x1w + y1w * y1w + z1w * z1w);
        wallContactOne(k, ra, va, wa, xiw, x1w, y1w, z1w, r1w, nst, df, dt);
        add3(FC, df);
        MC[0] += ra * dt[0];
        MC[1] += ra * dt[1];
        MC[2] += ra * dt[2];
        for (int c = 0; c < 3; ++c)
          if (df[c] != 0.0) atomicAdd(&acc[GA_WALL + 6 * w + c], -df[c]);
      }
    }
    // totals (src/DEM.cpp:745-762) and integration (:2681-2707)
    double FH[3], MH[3], FG[3];
    load3(a.FHydro, P, i, FH);
    load3(a.MHydro, P, i, MH);
    load3(a.FGrav, P, i, FG);
    double FT[3], MT[3];
    for (int c = 0; c < 3; ++c) {
      FT[c] = 0.0 + ((((FH[c] + FC[c]) + FL[c]) + FG[c]) + FR[c]);
      MT[c] = 0.0 + ((MH[c] + MC[c]) + ML[c]);
    }
    const double dtt = k.dt, im = a.invm[i], iI = a.invI[i];
    for (int c = 0; c < 3; ++c) {
      const double xn = xa[c] + (dtt * va[c] + dtt * dtt * FT[c] * im);
      a.x0[c * P + i] = xn;
      if (c == 1) {
        a.dispY[i] = a.xinitY[i] - xn;
        if (stepNo == k.objWaitTime) a.xinitY[i] = xn;
      }
      a.x1[c * P + i] = va[c] + dtt * FT[c] * im;
      a.w1[c * P + i] = wa[c] + dtt * MT[c] * iI;
      a.FContact[c * P + i] = FC[c];
      a.MContact[c * P + i] = MC[c];
      a.FLub[c * P + i] = FL[c];
      a.MLub[c * P + i] = ML[c];
      a.FRep[c * P + i] = FR[c];
      a.FTotal[c * P + i] = FT[c];
      a.MTotal[c * P + i] = MT[c];
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
