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

#include "kernels_decl.h"

namespace lbdem {

__device__ __forceinline__ int s_int(double x) { return x >= 0 ? (int)x : (int)(x - 1.0); }
__device__ __forceinline__ int n_int(double x) { return x >= 0 ? (int)(x + 0.5) : (int)(x - 0.5); }
__device__ __forceinline__ double boxf(double a, double b) { return a - s_int(a / b) * b; }
__device__ __forceinline__ double n_image(double a, double b) { return a - n_int(a / b) * b; }
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }


// ---- evalMaxDisp and the rebuild trigger -----------------------------------

// DEM::evalMaxDisp and the rebuild trigger of DEM::discreteElementStep
// (src/DEM.cpp:460-470, 368-378): the maximum of |x1|^2 over the particles
// (exact in any order: atomicMax on the bit patterns of non-negative
// doubles), then the last block to finish decides on a rebuild.
__global__ void __launch_bounds__(256) demBegin(Consts k, DemArgs a, int forceRebuild) {
  __shared__ double red[8];
  __shared__ bool last;
  double m = 0.0;
  const int P = k.nPart;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    const double vx = a.x1[i], vy = a.x1[P + i], vz = a.x1[2 * P + i];
    const double n2 = vx * vx + vy * vy + vz * vz;
    if (n2 > m) m = n2;
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

__global__ void nbrCellAssign(Consts k, DemArgs a) {
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
    atomicAdd(a.cellCount + l, 1);
  }
}

// exclusive scan of the cell counts (one CTA) and the occupancy check
__global__ void __launch_bounds__(1024) nbrCellScan(Consts k, DemArgs a) {
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

__global__ void nbrCellScatter(Consts k, DemArgs a) {
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
__global__ void nbrCellSort(Consts k, DemArgs a) {
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
                                          int P, int n1, int n2) {
  const double x12 = n_image(x0[n1] - x0[n2], k.demSize[0]);
  const double y12 = n_image(x0[P + n1] - x0[P + n2], k.demSize[1]);
  const double z12 = n_image(x0[2 * P + n1] - x0[2 * P + n2], k.demSize[2]);
  const double r12 = x12 * x12 + y12 * y12 + z12 * z12;
  const double cut = r[n1] + r[n2] + 2.0;
  return r12 <= cut * cut;
}

// New list of each particle: the events of the reference's cell sweep that
// involve it, sorted by (cell l1, neighbour-cell order, position of n1 in
// l1, position of n2 in l2) - the order in which the reference appends them.
__global__ void nbrBuildCells(Consts k, DemArgs a) {
  if (!a.iscal[IS_REBUILD] || a.iscal[IS_DIRECT]) return;
  const int cur = a.iscal[IS_LISTCUR];
  const int* oldList = a.list[cur];
  const double* oldXi = a.xi[cur];
  int* newList = a.list[1 - cur];
  double* newXi = a.xi[1 - cur];
  const int nlx = a.iscal[IS_NL], nly = a.iscal[IS_NL + 1], nlz = a.iscal[IS_NL + 2];
  const int P = k.nPart;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int cp = a.pcell[p];
    if (cp < 0) continue;
    const int cx = cp / (nly * nlz), cy = (cp / nlz) % nly, cz = cp % nlz;
    const int posp = a.ppos[p];
    unsigned long long keys[MAX_N];
    int nb[MAX_N];
    int cnt = 0;
    bool over = false;
    for (int kk = 0; kk < 27; ++kk) {
      const int dx = kk / 9 - 1, dy = (kk / 3) % 3 - 1, dz = kk % 3 - 1;
      // p as n1: partner q < p in l2 = l1 + d
      {
        const int l2 = ((cx + dx + nlx) % nlx) * nly * nlz + ((cy + dy + nly) % nly) * nlz +
                       (cz + dz + nlz) % nlz;
        const int s = a.cellStart[l2], n = a.cellFill[l2];
        for (int t = 0; t < n; ++t) {
          const int q = a.cellParts[s + t];
          if (q >= p || !nbrWithin(k, a.x0, a.r, P, p, q)) continue;
          if (cnt >= MAX_N - 1) { over = true; break; }
          keys[cnt] = ((unsigned long long)cp << 22) | ((unsigned long long)kk << 12) |
                      ((unsigned long long)posp << 6) | (unsigned long long)(t + 1);
          nb[cnt++] = q;
        }
      }
      // p as n2: partner q > p in l1 = l2 - d
      {
        const int l1 = ((cx - dx + nlx) % nlx) * nly * nlz + ((cy - dy + nly) % nly) * nlz +
                       (cz - dz + nlz) % nlz;
        const int s = a.cellStart[l1], n = a.cellFill[l1];
        for (int t = 0; t < n; ++t) {
          const int q = a.cellParts[s + t];
          if (q <= p || !nbrWithin(k, a.x0, a.r, P, q, p)) continue;
          if (cnt >= MAX_N - 1) { over = true; break; }
          keys[cnt] = ((unsigned long long)l1 << 22) | ((unsigned long long)kk << 12) |
                      ((unsigned long long)(t + 1) << 6) | (unsigned long long)posp;
          nb[cnt++] = q;
        }
      }
    }
    if (over) atomicOr(a.iscal + IS_ERROR, ERR_NBR_OVERFLOW);
    for (int i = 1; i < cnt; ++i) {
      const unsigned long long kv = keys[i];
      const int nv = nb[i];
      int j = i - 1;
      while (j >= 0 && keys[j] > kv) {
        keys[j + 1] = keys[j];
        nb[j + 1] = nb[j];
        --j;
      }
      keys[j + 1] = kv;
      nb[j + 1] = nv;
    }
    const int* ol = oldList + (long long)p * MAX_N;
    const double* ox = oldXi + (long long)p * 3 * MAX_N;
    int* nl = newList + (long long)p * MAX_N;
    double* nx = newXi + (long long)p * 3 * MAX_N;
    nl[0] = cnt;
    for (int s = 1; s <= cnt; ++s) nl[s] = nb[s - 1];
    // tangential history: last match in the old list wins; unmatched slots
    // keep their old value (src/DEM.cpp:633-651)
    const int ocnt = ol[0];
    for (int s = 1; s < MAX_N; ++s) {
      int src = s;
      if (s <= cnt)
        for (int l = 1; l <= ocnt; ++l)
          if (ol[l] == nl[s]) src = l;
      for (int c = 0; c < 3; ++c) nx[c * MAX_N + s] = ox[c * MAX_N + src];
    }
    for (int c = 0; c < 3; ++c) nx[c * MAX_N] = (double)cnt;
  }
}

// Direct-sum branch (src/DEM.cpp:515-554): lists in (n1, n2) order.
__global__ void nbrBuildDirect(Consts k, DemArgs a) {
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
__global__ void nbrDirectHistory(Consts k, DemArgs a) {
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
__global__ void nbrPartners(Consts k, DemArgs a) {
  if (!a.iscal[IS_REBUILD]) return;
  const int cur = 1 - a.iscal[IS_LISTCUR];
  const int* L = a.list[cur];
  const int P = k.nPart;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    const int* li = L + (long long)i * MAX_N;
    int* pt = a.partner + (long long)i * MAX_N;
    int* go = a.gorder + (long long)i * MAX_N;
    const int cnt = li[0];
    int ng = 0;
    for (int s = 1; s <= cnt; ++s)
      if (li[s] < i) go[ng++] = s;
    const int nown = ng;
    for (int s = 1; s <= cnt; ++s) {
      const int j = li[s];
      pt[s] = 0;
      if (j <= i) continue;
      int occ = 0;
      for (int t = 1; t < s; ++t)
        if (li[t] == j) ++occ;
      const int* lj = L + (long long)j * MAX_N;
      int seen = 0;
      for (int t = 1; t <= lj[0]; ++t)
        if (lj[t] == i) {
          if (seen == occ) {
            pt[s] = t;
            break;
          }
          ++seen;
        }
      go[ng++] = s;
    }
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
}

// Owner slots of the new lists (slot s of particle i with list[i][s] < i),
// so that the pair pass runs one thread per pair. The order of the entries
// does not matter: every pair writes only its own slot's outputs.
__global__ void nbrPairList(Consts k, DemArgs a) {
  if (!a.iscal[IS_REBUILD]) return;
  const int* L = a.list[1 - a.iscal[IS_LISTCUR]];
  const long long total = (long long)k.nPart * MAX_N;
  const int cap = max(k.nPart, 1) * (MAX_N / 2);
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(idx % MAX_N);
    if (s == 0) continue;
    const int i = (int)(idx / MAX_N);
    if (s > L[(long long)i * MAX_N] || L[idx] >= i) continue;
    const int pos = atomicAdd(a.iscal + IS_NPAIRS, 1);
    if (pos < cap) a.pairList[pos] = (int)idx;
    else atomicOr(a.iscal + IS_ERROR, ERR_NBR_OVERFLOW);
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

// DEM::calculateParticleContactForces, one pair (src/DEM.cpp:1506-1700)
__device__ void pairContact(const Consts& k, double ra, double rb, const double* xa,
                            const double* xb, const double* va, const double* vb,
                            const double* wa, const double* wb, double* xi, double* out) {
  const double rad = 0.5 * (ra + rb);
  const double x12 = xa[0] - xb[0], y12 = xa[1] - xb[1], z12 = xa[2] - xb[2];
  const double r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
  const double urx = va[0] - vb[0], ury = va[1] - vb[1], urz = va[2] - vb[2];
  const double nx = x12 / r12, ny = y12 / r12, nz = z12 / r12;
  const double gn = urx * nx + ury * ny + urz * nz;
  const double mu = k.mu, kk = k.k, c = k.c;
  const double del = 2 * rad - r12;
  double fnx, fny, fnz, ftx, fty, ftz;
  if (del > 0.0) {
    if (mu != 0.0) {
      const double ox = ra * wa[0] + rb * wb[0];
      const double oy = ra * wa[1] + rb * wb[1];
      const double oz = ra * wa[2] + rb * wb[2];
      const double vx = urx + ny * oz - nz * oy - gn * nx;
      const double vy = ury + nz * ox - nx * oz - gn * ny;
      const double vz = urz + nx * oy - ny * ox - gn * nz;
      const double xi12 = xi[0] * nx + xi[1] * ny + xi[2] * nz;
      xi[0] -= xi12 * nx;
      xi[1] -= xi12 * ny;
      xi[2] -= xi12 * nz;
      fnx = kk * del * nx - c * gn * nx;
      fny = kk * del * ny - c * gn * ny;
      fnz = kk * del * nz - c * gn * nz;
      const double kt = 0.2 * kk;
      const double dct = k.kinVisc == 0.0 ? c : 0.0;
      ftx = -kt * xi[0] - dct * vx;
      fty = -kt * xi[1] - dct * vy;
      ftz = -kt * xi[2] - dct * vz;
      const double fnn = sqrt(fnx * fnx + fny * fny + fnz * fnz);
      const double ftt = sqrt(ftx * ftx + fty * fty + ftz * ftz);
      const double fri = mu * fnn;
      const double tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
      xi[0] += vx * k.dt;
      xi[1] += vy * k.dt;
      xi[2] += vz * k.dt;
      if (fri < ftt) {
        ftx = fri * tx;
        fty = fri * ty;
        ftz = fri * tz;
        xi[0] = -(1 / kt) * (ftx + dct * vx);
        xi[1] = -(1 / kt) * (fty + dct * vy);
        xi[2] = -(1 / kt) * (ftz + dct * vz);
      }
    } else {
      fnx = kk * del * nx - c * gn * nx;
      fny = kk * del * ny - c * gn * ny;
      fnz = kk * del * nz - c * gn * nz;
      ftx = fty = ftz = 0.0;
    }
  } else {
    fnx = fny = fnz = ftx = fty = ftz = 0.0;
    xi[0] = xi[1] = xi[2] = 0.0;
  }
  out[0] = fnx + ftx;
  out[1] = fny + fty;
  out[2] = fnz + ftz;
  out[3] = fty * nz - ftz * ny;
  out[4] = ftz * nx - ftx * nz;
  out[5] = ftx * ny - fty * nx;
}

// Nguyen-Ladd lubrication of a sphere pair (src/DEM.cpp:2325-2491) or of a
// particle and an impactor (:1158-1323; same algebra with the impactor as
// sphere 2). Returns false outside the cut-off.
__device__ bool pairLub(const Consts& k, double ra, double rb, const double* xa,
                        const double* xb, const double* va, const double* vb, const double* wa,
                        const double* wb, double* out) {
  const double lub_N = k.lubN, lub_T = k.lubT, lub_R = k.lubR, cut = k.lubCut;
  const double rad = 0.5 * (ra + rb);
  double x12 = xa[0] - xb[0], y12 = xa[1] - xb[1], z12 = xa[2] - xb[2];
  const double r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
  const double umx = va[0] - vb[0], umy = va[1] - vb[1], umz = va[2] - vb[2];
  const double w1x = wa[0], w1y = wa[1], w1z = wa[2];
  const double w2x = wb[0], w2y = wb[1], w2z = wb[2];
  const double dr = r12 - 2.0 * rad;
  const double h = dmax(dr, cut);
  if (!(dr < dmax(cut, dmax(lub_N, dmax(lub_T, lub_R))))) return false;
  const double alpha = 3.14159265358979323846 * k.kinVisc * rad * k.dt;
  const double beta1 = rb / ra;
  const double beta2 = beta1 * beta1;
  const double beta3 = beta1 * beta2;
  const double beta4 = pow((1 + beta1), 4.0);
  double Xa, Ya, Yb1, Yb2, Yc11, Yc12, Yc21, Yc22, h_c, beta;
  if (dr < dmax(cut, lub_N)) {
    Xa = 4.0 * beta2 / beta4;
    h_c = dmax(dr, lub_N);
    Xa *= rad / h - rad / h_c;
    Xa *= 6.0 * alpha;
  } else {
    Xa = 0.0;
  }
  if (dr < dmax(cut, lub_T)) {
    Ya = 8.0 * beta1 * (2.0 + beta1 + 2.0 * beta2) / (15.0 * beta4);
    Yb1 = -4.0 * beta1 * (4.0 + beta1) / (5.0 * beta4);
    Yb2 = 4.0 * beta1 * (4.0 * beta2 + beta1) / (5.0 * beta4);
    h_c = dmax(dr, lub_T);
    beta = alpha * log(h_c / h);
    Ya *= 6.0 * beta;
    Yb1 *= 4.0 * beta * rad;
    Yb2 *= 4.0 * beta * rad;
  } else {
    Ya = Yb1 = Yb2 = 0.0;
  }
  if (dr < dmax(cut, lub_R)) {
    Yc11 = 16.0 * beta1 / (5.0 * beta4);
    Yc12 = 4.0 * beta2 / (5.0 * beta4);
    Yc21 = 4.0 * beta2 / (5.0 * beta4);
    Yc22 = 16.0 * beta3 / (5.0 * beta4);
    h_c = dmax(dr, lub_R);
    beta = alpha * log(h_c / h);
    Yc11 *= 8.0 * beta * rad * rad;
    Yc12 *= 8.0 * beta * rad * rad;
    Yc21 *= 8.0 * beta * rad * rad;
    Yc22 *= 8.0 * beta * rad * rad;
  } else {
    Yc11 = Yc12 = Yc21 = Yc22 = 0.0;
  }
  x12 /= r12;
  y12 /= r12;
  z12 /= r12;
  const double um_r = umx * x12 + umy * y12 + umz * z12;
  const double w1_r = w1x * x12 + w1y * y12 + w1z * z12;
  const double w2_r = w2x * x12 + w2y * y12 + w2z * z12;
  const double umxrx = umy * z12 - umz * y12;
  const double umxry = umz * x12 - umx * z12;
  const double umxrz = umx * y12 - umy * x12;
  const double w1xrx = w1y * z12 - w1z * y12;
  const double w1xry = w1z * x12 - w1x * z12;
  const double w1xrz = w1x * y12 - w1y * x12;
  const double w2xrx = w2y * z12 - w2z * y12;
  const double w2xry = w2z * x12 - w2x * z12;
  const double w2xrz = w2x * y12 - w2y * x12;
  double Fx = -Xa * um_r * x12 - Ya * (umx - um_r * x12);
  double Fy = -Xa * um_r * y12 - Ya * (umy - um_r * y12);
  double Fz = -Xa * um_r * z12 - Ya * (umz - um_r * z12);
  Fx += -Yb1 * w1xrx + Yb2 * w2xrx;
  Fy += -Yb1 * w1xry + Yb2 * w2xry;
  Fz += -Yb1 * w1xrz + Yb2 * w2xrz;
  double T1x = Yb1 * umxrx, T1y = Yb1 * umxry, T1z = Yb1 * umxrz;
  double T2x = -Yb2 * umxrx, T2y = -Yb2 * umxry, T2z = -Yb2 * umxrz;
  T1x += -Yc11 * (w1x - w1_r * x12) - Yc12 * (w2x - w2_r * x12);
  T1y += -Yc11 * (w1y - w1_r * y12) - Yc12 * (w2y - w2_r * y12);
  T1z += -Yc11 * (w1z - w1_r * z12) - Yc12 * (w2z - w2_r * z12);
  T2x += -Yc21 * (w1x - w1_r * x12) - Yc22 * (w2x - w2_r * x12);
  T2y += -Yc21 * (w1y - w1_r * y12) - Yc22 * (w2y - w2_r * y12);
  T2z += -Yc21 * (w1z - w1_r * z12) - Yc22 * (w2z - w2_r * z12);
  out[0] = Fx;
  out[1] = Fy;
  out[2] = Fz;
  out[3] = T1x;
  out[4] = T1y;
  out[5] = T1z;
  out[6] = T2x;
  out[7] = T2y;
  out[8] = T2z;
  return true;
}

// DEM::calculateParticleElectroForces, one pair (src/DEM.cpp:1413-1449)
__device__ void pairRep(const Consts& k, double ra, double rb, const double* xa,
                        const double* xb, double* out) {
  const double rad = 0.5 * (ra + rb);
  const double x12 = xa[0] - xb[0], y12 = xa[1] - xb[1], z12 = xa[2] - xb[2];
  const double r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
  const double nx = x12 / r12, ny = y12 / r12, nz = z12 / r12;
  const double del = 2 * rad - r12;
  if (del <= 0.0) {
    out[0] = k.electro * exp(del / k.debye) * nx;
    out[1] = k.electro * exp(del / k.debye) * ny;
    out[2] = k.electro * exp(del / k.debye) * nz;
  } else {
    out[0] = k.electro * nx;
    out[1] = k.electro * ny;
    out[2] = k.electro * nz;
  }
}

__device__ __forceinline__ void load3(const double* a, int P, int i, double* v) {
  v[0] = a[i];
  v[1] = a[P + i];
  v[2] = a[2 * P + i];
}

// Owner pass: every pair (n1 > n2) evaluated once from n1's slot, one
// thread per entry of the owner-pair list.
__global__ void demPairs(Consts k, DemArgs a) {
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
    double* out = a.pairbuf + (long long)idx * PAIR_VALS;
    uint8_t flag = 0;
    if (lubOn && pairLub(k, ra, rb, xa, xb, va, vb, wa, wb, out + 6)) flag |= 1;
    double xi[3] = {xii[s], xii[MAX_N + s], xii[2 * MAX_N + s]};
    pairContact(k, ra, rb, xa, xb, va, vb, wa, wb, xi, out);
    xii[s] = xi[0];
    xii[MAX_N + s] = xi[1];
    xii[2 * MAX_N + s] = xi[2];
    pairRep(k, ra, rb, xa, xb, out + 15);
    a.pairflag[idx] = flag;
  }
}

// ---- gather, walls, impactor, integration ------------------------------------

// Particle-wall contact (src/DEM.cpp:1956-2108) or the fictional lid
// (:2166-2292); returns the force and torque arm; updates xiw.
__device__ void wallContactOne(const Consts& k, double r, const double* x, const double* v,
                               const double* w, double* xiw, double x1w, double y1w,
                               double z1w, double* nstale, double* df, double* dt) {
  const double r1w = sqrt(x1w * x1w + y1w * y1w + z1w * z1w);
  const double delw = r - r1w;
  double fnx, fny, fnz, ftx, fty, ftz;
  if (delw > 0.0) {
    nstale[0] = x1w / r1w;
    nstale[1] = y1w / r1w;
    nstale[2] = z1w / r1w;
    const double nx = nstale[0], ny = nstale[1], nz = nstale[2];
    const double urx = v[0], ury = v[1], urz = v[2];
    const double gn = urx * nx + ury * ny + urz * nz;
    if (k.mu != 0.0) {
      const double ox = r * w[0], oy = r * w[1], oz = r * w[2];
      const double vx = urx + ny * oz - nz * oy - gn * nx;
      const double vy = ury + nz * ox - nx * oz - gn * ny;
      const double vz = urz + nx * oy - ny * ox - gn * nz;
      const double xi = xiw[0] * nx + xiw[1] * ny + xiw[2] * nz;
      xiw[0] -= xi * nx;
      xiw[1] -= xi * ny;
      xiw[2] -= xi * nz;
      fnx = k.k * delw * nx - k.c * gn * nx;
      fny = k.k * delw * ny - k.c * gn * ny;
      fnz = k.k * delw * nz - k.c * gn * nz;
      const double kt = 0.2 * k.k;
      const double dct = k.kinVisc == 0.0 ? k.c : 0.0;
      ftx = -kt * xiw[0] - dct * vx;
      fty = -kt * xiw[1] - dct * vy;
      ftz = -kt * xiw[2] - dct * vz;
      const double fnn = sqrt(fnx * fnx + fny * fny + fnz * fnz);
      const double ftt = sqrt(ftx * ftx + fty * fty + ftz * ftz);
      const double fri = k.mu * fnn;
      const double tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
      xiw[0] += vx * k.dt;
      xiw[1] += vy * k.dt;
      xiw[2] += vz * k.dt;
      if (fri < ftt) {
        ftx = fri * tx;
        fty = fri * ty;
        ftz = fri * tz;
        xiw[0] = -(1 / kt) * (ftx + dct * vx);
        xiw[1] = -(1 / kt) * (fty + dct * vy);
        xiw[2] = -(1 / kt) * (ftz + dct * vz);
      }
    } else {
      fnx = k.k * delw * nx - k.c * gn * nx;
      fny = k.k * delw * ny - k.c * gn * ny;
      fnz = k.k * delw * nz - k.c * gn * nz;
      ftx = fty = ftz = 0.0;
    }
  } else {
    fnx = fny = fnz = ftx = fty = ftz = 0.0;
    xiw[0] = xiw[1] = xiw[2] = 0.0;
  }
  df[0] = fnx + ftx;
  df[1] = fny + fty;
  df[2] = fnz + ftz;
  dt[0] = fty * nstale[2] - ftz * nstale[1];
  dt[1] = ftz * nstale[0] - ftx * nstale[2];
  dt[2] = ftx * nstale[1] - fty * nstale[0];
}

// Particle-wall lubrication (src/DEM.cpp:2541-2670)
__device__ bool wallLubOne(const Consts& k, double rad, const double* v, const double* w,
                           double x12, double y12, double z12, double* F, double* T) {
  const double cut = k.lubCut, lub_N = k.lubN, lub_T = k.lubT, lub_R = k.lubR;
  const double r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
  const double umx = v[0], umy = v[1], umz = v[2];
  const double w1x = w[0], w1y = w[1], w1z = w[2];
  const double dr = r12 - rad;
  const double h = dmax(dr, cut);
  if (!(dr < dmax(cut, dmax(lub_N, dmax(lub_T, lub_R))))) return false;
  const double alpha = 3.14159265358979323846 * k.kinVisc * rad * k.dt;
  double Xa, Ya, Yb1, Yc11, h_c, beta;
  if (dr < dmax(cut, lub_N)) {
    Xa = 1.0;
    h_c = dmax(dr, lub_N);
    Xa *= rad / h - rad / h_c;
    Xa *= 6.0 * alpha;
  } else {
    Xa = 0.0;
  }
  if (dr < dmax(cut, lub_T)) {
    Ya = 8.0 / 15.0;
    Yb1 = -1.0 / 5.0;
    h_c = dmax(dr, lub_T);
    beta = alpha * log(h_c / h);
    Ya *= 6.0 * beta;
    Yb1 *= 4.0 * beta * rad;
  } else {
    Ya = Yb1 = 0.0;
  }
  if (dr < dmax(cut, lub_R)) {
    Yc11 = 2.0 / 5.0;
    h_c = dmax(dr, lub_R);
    beta = alpha * log(h_c / h);
    Yc11 *= 8.0 * beta * rad * rad;
  } else {
    Yc11 = 0.0;
  }
  x12 /= r12;
  y12 /= r12;
  z12 /= r12;
  const double um_r = umx * x12 + umy * y12 + umz * z12;
  const double w1_r = w1x * x12 + w1y * y12 + w1z * z12;
  const double umxrx = umy * z12 - umz * y12;
  const double umxry = umz * x12 - umx * z12;
  const double umxrz = umx * y12 - umy * x12;
  const double w1xrx = w1y * z12 - w1z * y12;
  const double w1xry = w1z * x12 - w1x * z12;
  const double w1xrz = w1x * y12 - w1y * x12;
  F[0] = -Xa * x12 * um_r - Ya * (umx - um_r * x12);
  F[1] = -Xa * y12 * um_r - Ya * (umy - um_r * y12);
  F[2] = -Xa * z12 * um_r - Ya * (umz - um_r * z12);
  F[0] += -Yb1 * w1xrx;
  F[1] += -Yb1 * w1xry;
  F[2] += -Yb1 * w1xrz;
  T[0] = Yb1 * umxrx;
  T[1] = Yb1 * umxry;
  T[2] = Yb1 * umxrz;
  T[0] += -Yc11 * (w1x - w1_r * x12);
  T[1] += -Yc11 * (w1y - w1_r * y12);
  T[2] += -Yc11 * (w1z - w1_r * z12);
  return true;
}

// Particle-impactor contact (src/DEM.cpp:921-1090); dampCoeffTanw is an
// uninitialised local in the reference, zero under the pinned build.
__device__ void objContactOne(const Consts& k, double ra, double ro, const double* xa,
                              const double* xo, const double* va, const double* vo,
                              const double* wa, const double* wo, double* xio, double* df,
                              double* dt) {
  const double radw = 0.5 * (ra + ro);
  const double x1w = xa[0] - xo[0], y1w = xa[1] - xo[1], z1w = xa[2] - xo[2];
  const double r1w = sqrt(x1w * x1w + y1w * y1w + z1w * z1w);
  const double nx = x1w / r1w, ny = y1w / r1w, nz = z1w / r1w;
  const double urx = va[0] - vo[0], ury = va[1] - vo[1], urz = va[2] - vo[2];
  const double delw = (2 * radw) - r1w;
  const double dampCoeffTanw = 0.0;
  double fnx, fny, fnz, ftx, fty, ftz;
  if (delw > 0.0) {
    const double gn = urx * nx + ury * ny + urz * nz;
    if (k.mu != 0.0) {
      const double ox = ra * wa[0] + ro * wo[0];
      const double oy = ra * wa[1] + ro * wo[1];
      const double oz = ra * wa[2] + ro * wo[2];
      const double vx = urx + ny * oz - nz * oy - gn * nx;
      const double vy = ury + nz * ox - nx * oz - gn * ny;
      const double vz = urz + nx * oy - ny * ox - gn * nz;
      const double xi = xio[0] * nx + xio[1] * ny + xio[2] * nz;
      xio[0] -= xi * nx;
      xio[1] -= xi * ny;
      xio[2] -= xi * nz;
      fnx = k.k * delw * nx - k.c * gn * nx;
      fny = k.k * delw * ny - k.c * gn * ny;
      fnz = k.k * delw * nz - k.c * gn * nz;
      const double kt = 0.2 * k.k;
      ftx = -kt * xio[0];
      fty = -kt * xio[1];
      ftz = -kt * xio[2];
      const double fnn = sqrt(fnx * fnx + fny * fny + fnz * fnz);
      const double ftt = sqrt(ftx * ftx + fty * fty + ftz * ftz);
      const double fri = k.mu * fnn;
      const double tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
      if (fri < ftt) {
        ftx = fri * tx;
        fty = fri * ty;
        ftz = fri * tz;
        xio[0] = -(1 / kt) * (ftx + dampCoeffTanw * vx);
        xio[1] = -(1 / kt) * (fty + dampCoeffTanw * vy);
        xio[2] = -(1 / kt) * (ftz + dampCoeffTanw * vz);
      } else {
        xio[0] += vx * k.dt;
        xio[1] += vy * k.dt;
        xio[2] += vz * k.dt;
      }
    } else {
      fnx = k.k * delw * nx - k.c * gn * nx;
      fny = k.k * delw * ny - k.c * gn * ny;
      fnz = k.k * delw * nz - k.c * gn * nz;
      ftx = fty = ftz = 0.0;
    }
  } else {
    fnx = fny = fnz = ftx = fty = ftz = 0.0;
    xio[0] = xio[1] = xio[2] = 0.0;
  }
  df[0] = fnx + ftx;
  df[1] = fny + fty;
  df[2] = fnz + ftz;
  dt[0] = fty * nz - ftz * ny;
  dt[1] = ftz * nx - ftx * nz;
  dt[2] = ftx * ny - fty * nx;
}

__device__ __forceinline__ void add3(double* a, const double* b) {
  a[0] += b[0];
  a[1] += b[1];
  a[2] += b[2];
}
__device__ __forceinline__ void sub3(double* a, const double* b) {
  a[0] -= b[0];
  a[1] -= b[1];
  a[2] -= b[2];
}

// per-block shared accumulators for the impactor and wall sums
enum { GA_OBJ = 0, GA_WALL = GA_OBJ + 12 * MAX_OBJ, GA_N = GA_WALL + 6 * MAX_WALL };

// Impactor totals and integration, wall totals (src/DEM.cpp:773-790,
// 2742-2760), by the last block of demGather once every block's impactor
// and wall sums are in.
__device__ void demObjectsTail(const Consts& k, DemArgs& a) {
  const int stepNo = a.iscal[IS_DEMSTEP];
  const int o = threadIdx.x;
  // volatile: the sums other blocks added must not come from a line this
  // block's L1 cached earlier in the kernel
  if (o < k.nObj) {
    volatile double* ob = a.obj + o * OB_STRIDE;
    const double dtt = k.dt;
    for (int c = 0; c < 3; ++c) {
      ob[OB_FTOTAL + c] =
          0.0 + ((((ob[OB_FHYDRO + c] + ob[OB_FCONTACT + c]) + ob[OB_FLUB + c]) + ob[OB_FGRAV + c]) +
                 0.0);
      ob[OB_MTOTAL + c] = 0.0 + ((ob[OB_MHYDRO + c] + ob[OB_MCONTACT + c]) + ob[OB_MLUB + c]);
    }
    if (stepNo >= k.objWaitTime)
      for (int c = 0; c < 3; ++c) {
        const double x1 = ob[OB_X1 + c];
        ob[OB_X0 + c] += dtt * x1 + dtt * dtt * ob[OB_FTOTAL + c] * ob[OB_INVM];
        ob[OB_X1 + c] = x1 + dtt * ob[OB_FTOTAL + c] * ob[OB_INVM];
        ob[OB_W1 + c] += dtt * ob[OB_MTOTAL + c] * ob[OB_INVI];
      }
  }
  if (o < k.nWall) {
    volatile double* w = a.wallF + o * 12;
    for (int c = 0; c < 3; ++c) w[9 + c] = 0.0 + (((w[c] + w[3 + c]) + w[6 + c]) + 0.0);
  }
}

__global__ void __launch_bounds__(128) demGather(Consts k, DemArgs a) {
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
        double F[3], T[3];
        if (wallLubOne(k, ra, va, wa, x12, y12, z12, F, T)) {
          add3(FL, F);
          add3(ML, T);
          for (int c = 0; c < 3; ++c)
            if (F[c] != 0.0) atomicAdd(&acc[GA_WALL + 6 * w + 3 + c], -F[c]);
        }
      }
      for (int o = 0; o < k.nObj; ++o) {
        const double* ob = a.obj + o * OB_STRIDE;
        objContactOne(k, ra, ob[OB_R], xa, ob + OB_X0, va, ob + OB_X1, wa, ob + OB_W1, xio,
                      df, dt);
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
        if (pairLub(k, ra, ob[OB_R], xa, ob + OB_X0, va, ob + OB_X1, wa, ob + OB_W1, lo)) {
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
      wallContactOne(k, ra, xa, va, wa, xiw, 0.0, xa[1] - (k.demSize[1] - 0.3), 0.0, nst, df,
                     dt);
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
        wallContactOne(k, ra, xa, va, wa, xiw, x1w, y1w, z1w, nst, df, dt);
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
      a.x0[c * P + i] = xa[c] + (dtt * va[c] + dtt * dtt * FT[c] * im);
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
