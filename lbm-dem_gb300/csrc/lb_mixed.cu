// Mixed-precision lattice step: FP32 deviation storage (f - w, 76 B per
// node per lattice), FP32 collision with the reference's BGK + Guo forcing
// and particle coupling, push streaming with the reference's boundary rules
// rewritten for deviations. Interface masses, the free-surface mass budget
// and all DEM state stay FP64; the per-particle coupling sums are float
// partial sums converted once per particle (lbFinalizeKernel).
//
// Reference: LB::latticeBolzmannStep (src/LB.cpp:400-418) with
// node::reconstruct/shiftVelocity/computeEquilibrium/solveCollision/addForce
// (src/node.cpp:75-207), LB::computeHydroForces (src/LB.cpp:1901-1978) and
// LB::streaming (src/LB.cpp:1334-1544). In deviation form (initDensity = 1):
//   gas neighbour:     g_opp = -g_j + w_j (9 (c_j.u)^2 - 3 u^2)
//   static wall:       g_opp = g_j,           force 2 g_j c_j
//   moving object:     g_opp = g_j - BBi,     force (2 g_j - BBi) c_j
// This file is compiled without implicit FMA contraction; the collision uses
// explicit fused multiply-adds (lattice_common.cuh).
//
// Layout of the work: one warp handles 32 consecutive nodes of the x-major
// lattice per iteration of a grid-stride loop. The 18 streaming links are
// resolved in an unrolled loop that only knows "active neighbour" and "gas
// neighbour"; links to walls, slip walls and impactors are marked and
// handled afterwards in one non-unrolled loop, which keeps the hot loop
// small enough for the instruction caches.
#include "lattice_common.cuh"

namespace lbdem {

namespace {

// direction j packed for the dynamic-index boundary path:
// bits 0-1 cx+1, 2-3 cy+1, 4-5 cz+1, 8-12 opposite direction
__host__ __device__ constexpr int packDir(int j) {
  return (CX(j) + 1) | ((CY(j) + 1) << 2) | ((CZ(j) + 1) << 4) | (OPPJ(j) << 8);
}
__constant__ int c_dir[Q] = {packDir(0),  packDir(1),  packDir(2),  packDir(3),  packDir(4),
                             packDir(5),  packDir(6),  packDir(7),  packDir(8),  packDir(9),
                             packDir(10), packDir(11), packDir(12), packDir(13), packDir(14),
                             packDir(15), packDir(16), packDir(17), packDir(18)};

constexpr unsigned FULL = 0xffffffffu;
constexpr unsigned ALL_LINKS = 0x7FFFEu;  // bits 1..18
// neighbour types whose link needs no fix-up after the unrolled streaming
// loop: fluid 0, gas 2, interface 3, slip walls 5/6 (their diagonal links'
// slip rule follows the step, slipStash / slipApply), walls 7/8, topography 11
constexpr unsigned PLAIN_TYPES = (1u << 0) | (1u << 2) | (1u << 3) | (1u << 5) | (1u << 6) |
                                 (1u << 7) | (1u << 8) | (1u << 11);

// ---- asynchronous bulk copies into shared memory (cp.async.bulk) tracked
// by mbarriers; every wait is bounded ----
constexpr int WAIT_LIMIT = 1 << 22;  // try_wait rounds before a wait gives up

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbarInit(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count)
               : "memory");
}
// make the initialised barriers visible to the async proxy
__device__ __forceinline__ void fenceBarrierInit() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbarExpectTx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbarArrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(bar)) : "memory");
}
__device__ __forceinline__ bool mbarTryWait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smemAddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// with LBDEM_DEBUG_NO_LATTICE_COPIES no copy is ever issued, so nothing can
// be in flight when a wait gives up and a short limit is safe
constexpr int WAIT_LIMIT_NO_COPIES = 1 << 14;
// one thread waits for the phase of the given parity to complete
__device__ __forceinline__ bool mbarWait(uint64_t* bar, unsigned parity) {
  for (int it = 0; it < WAIT_LIMIT; ++it)
    if (mbarTryWait(bar, parity)) return true;
  return false;
}
// all lanes of a warp wait together; the result is warp-uniform
__device__ __forceinline__ bool warpWait(uint64_t* bar, unsigned parity, int limit) {
  for (int it = 0; it < limit; ++it)
    if (__all_sync(0xffffffffu, mbarTryWait(bar, parity))) return true;
  return false;
}
// global -> shared bulk copy; both addresses 16-byte aligned, bytes % 16 == 0
__device__ __forceinline__ void bulkLoad(void* dst, const void* src, unsigned bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smemAddr(dst)), "l"(src), "r"(bytes), "r"(smemAddr(bar))
      : "memory");
}

// Segmented reduction of the particle coupling terms over runs of
// consecutive lanes that share a particle index and a lattice row, then one
// set of float atomics per run (issued by the run heads together) into the
// particle's 64-byte line of sums.
//
// Per run only 7 sums are needed: D = sum d, L = sum o d with o the lane's
// offset from the run head, and V = sum massOld. With r the node position
// relative to the particle centre, r_y and r_z are the same for every node
// of a run and r_x = r_x(head) + o, so
//   R_ab = sum r_a d_b:  R_xb = L_b + r_x(head) D_b,  R_yb = r_y D_b,
//   R_zb = r_z D_b.
// The accumulators hold D (3), R (9, row-major a*3+b) and V; the torque
// (antisymmetric part of R) and the stresslet (R scaled) are formed per
// particle in lbFinalizeKernel.
__device__ __forceinline__ void particleRunReduce(int key, int ix, float dx, float dy, float dz,
                                                  float rx, float ry, float rz, float massOld,
                                                  float* acc) {
  const int lane = threadIdx.x & 31;
  const unsigned pm = __ballot_sync(FULL, key >= 0);
  const int prevKey = __shfl_up_sync(FULL, key, 1);
  const bool head = key >= 0 && (lane == 0 || prevKey != key || ix == 0);
  const unsigned hm = __ballot_sync(FULL, head);
  const unsigned stop = hm | ~pm;
  const unsigned upto = lane == 31 ? FULL : (2u << lane) - 1u;  // lanes 0..lane
  const unsigned above = stop & ~upto;
  const int end = above ? __ffs(above) - 1 : 32;
  const int headLane = 31 - __clz(hm & upto);  // meaningful for key >= 0
  const int maxLen = (int)__reduce_max_sync(FULL, head ? (unsigned)(end - lane) : 0u);
  const float o = key >= 0 ? (float)(lane - headLane) : 0.0f;
  float v[7] = {dx, dy, dz, o * dx, o * dy, o * dz, massOld};
  for (int st = 1; st < maxLen; st <<= 1) {
    const bool take = lane + st < end;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      const float t = __shfl_down_sync(FULL, v[i], st);
      if (take) v[i] += t;
    }
  }
  if (head) {
    // the particle's line is 64-byte aligned: three 16-byte vector
    // reductions and one scalar instead of thirteen scalar atomics
    float* q = acc + (size_t)key * ACCF_STRIDE;
    float4* q4 = reinterpret_cast<float4*>(q);
    atomicAdd(q4, make_float4(v[0], v[1], v[2], __fmaf_rn(rx, v[0], v[3])));
    atomicAdd(q4 + 1, make_float4(__fmaf_rn(rx, v[1], v[4]), __fmaf_rn(rx, v[2], v[5]),
                                  ry * v[0], ry * v[1]));
    atomicAdd(q4 + 2, make_float4(ry * v[2], rz * v[0], rz * v[1], rz * v[2]));
    atomicAdd(q + 12, v[6]);
  }
}

}  // namespace

LBDEM_KERNEL(MIXED_BOUNDS, lbStepMixed, LbArgs, lb) {
  extern __shared__ __align__(128) unsigned char stageMem[];  // MIXED_STAGES x stage
  __shared__ uint64_t fullBar[MIXED_STAGES], emptyBar[MIXED_STAGES];
  __shared__ int abortFlag;
  __shared__ float accO[6 * MAX_OBJ];
  __shared__ float sObj[6 * MAX_OBJ];  // impactor centre (x0/L) and velocity (x1/S)
  __shared__ double accX;
  __shared__ int sbox[6];
  __shared__ unsigned scnt[2];
  __shared__ int4 stageHdr[MIXED_STAGES];        // chunk index and its first node's x, y, z
  __shared__ uint8_t sAct[MIXED_MAX_MINE];       // warp activity bits of this block's chunks
  __shared__ uint16_t sList[MIXED_MAX_MINE];     // which of them to process
  __shared__ unsigned sCount;
  __shared__ unsigned sConsumed;  // iterations every consumer warp finished
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int st = 0; st < MIXED_STAGES; ++st) {
      mbarInit(&fullBar[st], 1);                  // thread 0's expect_tx
      mbarInit(&emptyBar[st], MIXED_CONSUMERS / 32);  // one arrival per consumer warp
    }
    abortFlag = 0;
    sConsumed = ~0u;
    fenceBarrierInit();
  }
  for (int i = tid; i < 6 * MAX_OBJ; i += blockDim.x) accO[i] = 0.0f;
  if (tid < k.nObj) {
    const double* ob = a.obj + tid * OB_STRIDE;
    for (int c = 0; c < 3; ++c) {
      sObj[6 * tid + c] = (float)(ob[OB_X0 + c] / k.uLength);
      sObj[6 * tid + 3 + c] = (float)(ob[OB_X1 + c] / k.uSpeed);
    }
  }
  if (tid < 3) sbox[tid] = INT_MAX;
  else if (tid < 6) sbox[tid] = -1;
  if (tid == 0) {
    accX = 0.0;
    scnt[0] = scnt[1] = 0u;
  }
  __syncthreads();
  const float* __restrict__ gin = (const float*)a.fin;
  float* __restrict__ gout = (float*)a.fout;
  const uint8_t* mk = a.mask;
  // node indices fit 32 bits (checked when the run is created)
  const unsigned N = (unsigned)k.N;
  const size_t NN = (size_t)k.N;    // stride of the interface arrays uS, hS
  const size_t NP = (size_t)k.NP;   // population plane stride (multiple of the chunk)
  const unsigned nChunks = (unsigned)(k.NP / MIXED_CHUNK);
  // chunks of this block: blockIdx.x, blockIdx.x + gridDim.x, ...
  const unsigned nMine =
      nChunks > blockIdx.x ? (nChunks - 1u - blockIdx.x) / gridDim.x + 1u : 0u;
  auto chunkOf = [&](unsigned it) { return blockIdx.x + it * gridDim.x; };
  const int lane = tid & 31;
  const int warp = tid >> 5;
  // Chunks with no active node are skipped: their activity bits (kept by
  // this kernel and set by whatever activates a node in between) are read
  // once, and warp 0 compacts the list of chunks to process.
  const bool useList = k.chunkAct != nullptr && nMine <= (unsigned)MIXED_MAX_MINE;
  if (useList) {
    for (unsigned it = tid; it < nMine; it += blockDim.x)
      sAct[it] = (uint8_t)k.chunkAct[chunkOf(it)];
    __syncthreads();
    if (warp == 0) {
      unsigned run = 0;
      for (unsigned b = 0; b < nMine; b += 32) {
        const unsigned it = b + lane;
        const bool on = it < nMine && sAct[it] != 0;
        const unsigned bal = __ballot_sync(FULL, on);
        if (on) sList[run + __popc(bal & ((1u << lane) - 1u))] = (uint16_t)it;
        run += __popc(bal);
      }
      if (lane == 0) sCount = run;
    }
    __syncthreads();
  }
  const unsigned nIter = useList ? sCount : nMine;
  double extra = 0.0;
  unsigned nact = 0, nif = 0;
  // The stage ring: bulk copies of the 19 population planes, solid indices,
  // densities and mask bytes of a chunk, completing on the stage's full
  // barrier. The producer warp issues iteration q once every consumer warp
  // has released iteration q - MIXED_STAGES (empty barrier); without it,
  // thread 0 issues iterations 0 .. MIXED_STAGES-1 up front and iteration
  // i + MIXED_STAGES - 1 at its iteration i once every warp has released
  // iteration i - 1.
  auto issue = [&](unsigned q) {
    const int st = (int)(q % MIXED_STAGES);
    unsigned char* sb = stageMem + st * MIXED_STAGE_BYTES;
    const unsigned c = chunkOf(useList ? sList[q] : q);
    const size_t off = (size_t)c * MIXED_CHUNK;
    int cx0, cy0, cz0;
    coords(k, (long long)off, cx0, cy0, cz0);
    stageHdr[st] = make_int4((int)c, cx0, cy0, cz0);
    mbarExpectTx(&fullBar[st], MIXED_STAGE_BYTES);
#pragma unroll 1
    for (int j = 0; j < Q; ++j)
      bulkLoad(sb + j * MIXED_CHUNK * 4, gin + j * NP + off, MIXED_CHUNK * 4, &fullBar[st]);
    if (LBDEM_MIXED_STAGE_SIDE) {
      bulkLoad(sb + MIXED_STAGE_SOLID, a.solid + off, MIXED_CHUNK * 4, &fullBar[st]);
      bulkLoad(sb + MIXED_STAGE_NF, a.nF + off, MIXED_CHUNK * 4, &fullBar[st]);
    }
    bulkLoad(sb + MIXED_STAGE_MASK, mk + off, MIXED_CHUNK, &fullBar[st]);
  };
  unsigned issued = 0;  // meaningful in thread 0
  // test of the timeout path: no copy is issued, every wait runs out
  const bool noCopies = (k.debugFlags & LBDEM_DEBUG_NO_LATTICE_COPIES) != 0;
  const int waitLimit = noCopies ? WAIT_LIMIT_NO_COPIES : WAIT_LIMIT;
  const int X = k.X, Y = k.Y, sy = (int)k.sy, sz = (int)k.sz;
  unsigned i = 0;
#if LBDEM_MIXED_PRODUCER
  // the producer warp keeps the ring full: iteration q is issued once every
  // consumer warp has released iteration q - MIXED_STAGES of the same stage
  if (warp == MIXED_CONSUMERS / 32) {
    if (lane == 0 && !noCopies) {
      for (; issued < nIter; ++issued) {
        if (*(volatile int*)&abortFlag) break;
        if (issued >= (unsigned)MIXED_STAGES) {
          const unsigned pq = issued - (unsigned)MIXED_STAGES;
          if (!mbarWait(&emptyBar[pq % MIXED_STAGES], (pq / MIXED_STAGES) & 1u)) {
            atomicOr(a.iscal + IS_ERROR, ERR_PIPELINE);
            abortFlag = 1;
            break;
          }
        }
        issue(issued);
      }
    }
    i = nIter;  // the producer consumes nothing
  }
#else
  if (tid == 0 && !noCopies)
    for (; issued < nIter && issued < (unsigned)MIXED_STAGES; ++issued) issue(issued);
#endif
  for (; i < nIter; ++i) {
    const int st = (int)(i % MIXED_STAGES);
    const unsigned ph = (i / MIXED_STAGES) & 1u;
    if (__any_sync(FULL, *(volatile int*)&abortFlag != 0) || !warpWait(&fullBar[st], ph, waitLimit)) {
      if (lane == 0) {
        atomicOr(a.iscal + IS_ERROR, ERR_PIPELINE);
        abortFlag = 1;
      }
      break;
    }
    const unsigned char* sb = stageMem + st * MIXED_STAGE_BYTES;
    const int4 hdr = stageHdr[st];
    const unsigned c = (unsigned)hdr.x;
    const unsigned x = c * MIXED_CHUNK + tid;
    const bool valid = x < N;
    // this thread's node coordinates from the chunk's first node
    int ix = hdr.y + tid, iy = hdr.z, iz = hdr.w;
    while (ix >= X) {
      ix -= X;
      if (++iy >= Y) {
        iy = 0;
        ++iz;
      }
    }
    float g[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) g[j] = ((const float*)sb)[j * MIXED_CHUNK + tid];
    const uint8_t m = valid ? sb[MIXED_STAGE_MASK + tid] : (uint8_t)2;
    const uint32_t sol = LBDEM_MIXED_STAGE_SIDE ? ((const uint32_t*)(sb + MIXED_STAGE_SOLID))[tid]
                         : ((valid && (m & PFLAG)) ? __ldg(a.solid + x) : 0u);
    const int t = m & TYPE_MASK;
    const bool act = valid && isActiveT(t);
    // particle nodes: their particle's kinematics and old mass, loaded first
    const bool coupled = act && (m & PFLAG) && sol < (uint32_t)k.nPart;
    KinF kin{};
    float massOld = 0.0f;
    if (coupled) {
      kin = loadKinF(a.pkf, sol);
      massOld = t == 3 ? (float)a.mass[x]
                : LBDEM_MIXED_STAGE_SIDE ? ((const float*)(sb + MIXED_STAGE_NF))[tid] : a.nF[x];
    }
    __syncwarp();
    if (lane == 0) mbarArrive(&emptyBar[st]);  // this warp is done with the stage
    if (!LBDEM_MIXED_PRODUCER && tid == 0 && i >= 1 && issued < nIter && !noCopies) {
      // refill the stage of iteration i - 1 with iteration i - 1 + MIXED_STAGES
      const unsigned pi = i - 1u;
      if (mbarWait(&emptyBar[pi % MIXED_STAGES], (pi / MIXED_STAGES) & 1u)) {
        issue(issued);
        ++issued;
      } else {
        atomicOr(a.iscal + IS_ERROR, ERR_PIPELINE);
        abortFlag = 1;
      }
    }
    // cleanLists (ABIT) and the neighbour cache (BULK) of this node
    uint8_t nm = (uint8_t)(m & ~(ABIT | BULK));
    if (__any_sync(FULL, act)) {
      unsigned actN = ALL_LINKS, gasN = 0, spcN = 0, wallN = 0;
      NodeStateF s;
      s.dx = s.dy = s.dz = s.rx = s.ry = s.rz = 0.0f;
      int key = -1;
      if (act) {
        // links into the box's wall layer, known from the coordinates
        wallN = boxWallLinks(k, ix, iy, iz);
        if (m & BULK) {
          actN = ALL_LINKS & ~wallN;
        } else {
          actN = 0;
#pragma unroll
          for (int j = 1; j < Q; ++j) {
            const int tl = mk[x + (unsigned)k.nbOff[j]] & TYPE_MASK;
            actN |= (unsigned)isActiveT(tl) << j;
            gasN |= (unsigned)(tl == 2) << j;
            spcN |= ((PLAIN_TYPES >> tl) & 1u ^ 1u) << j;
          }
        }
        nm |= (uint8_t)(ABIT | ((actN | wallN) == ALL_LINKS ? BULK : 0));
        collideNodeMixed(k, g, coupled, kin, massOld, ix, iy, iz, s);
        if (coupled) key = (int)sol;
        else if (m & PFLAG) atomicOr(a.iscal + IS_ERROR, ERR_PARTICLE_INDEX);
      }
      if (__any_sync(FULL, key >= 0))
        particleRunReduce(key, ix, s.dx, s.dy, s.dz, s.rx, s.ry, s.rz, massOld, a.pAccF);
      // Warps whose active nodes link only to active nodes and to the box's
      // wall layer skip the per-link tests: every population is pushed (a
      // push into the wall layer lands in a wall node's slot, which no step
      // reads and no other node writes), then the wall links bounce back.
      // The first and last warps of every lattice row are of this kind.
      const bool pushAll = __all_sync(FULL, !act || (actN | wallN) == ALL_LINKS);
      if (act) {
        ++nact;
        __stcs(gout + x, g[0]);
      }
      if (pushAll) {
        if (act) {
#pragma unroll
          for (int j = 1; j < Q; ++j) __stcs(gout + (x + k.pushOff[j]), g[j]);
          if (wallN) {
#pragma unroll
            for (int j = 1; j < Q; ++j)
              if ((wallN >> j) & 1u) gout[OPPJ(j) * NP + x] = g[j];
          }
        }
      } else if (act) {
        const float usq3 = 3.0f * __fmaf_rn(s.ux, s.ux, __fmaf_rn(s.uy, s.uy, s.uz * s.uz));
#pragma unroll
        for (int j = 1; j < Q; ++j) {
          if ((actN >> j) & 1u) {
            __stcs(gout + (x + k.pushOff[j]), g[j]);
          } else {
            float out = g[j];
            if ((gasN >> j) & 1u) {
              const float vu = dotcf(j, s.ux, s.uy, s.uz);
              out = __fmaf_rn((float)WJ(j), __fmaf_rn(9.0f * vu, vu, -usq3), -g[j]);
            }
            gout[OPPJ(j) * NP + x] = out;
          }
        }
        // impactor links and unexpected types: the value stored above is
        // g_j; fix it up and add the link forces. Walls (plain bounce-back)
        // get their force from lbWallForceMixed after this kernel.
        unsigned special = spcN;
        if (special) {
          float fo[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
          int ocur = -1;
#pragma unroll 1
          for (; special; special &= special - 1u) {
            const int j = __ffs(special) - 1;
            const int dj = c_dir[j];
            const int cx = (dj & 3) - 1, cy = ((dj >> 2) & 3) - 1, cz = ((dj >> 4) & 3) - 1;
            const unsigned lk = x + (unsigned)(cx + cy * sy + cz * sz);
            const uint8_t mlk = mk[lk];
            const int tl = mlk & TYPE_MASK;
            const int oi = a.objIdx[lk];
            if (tl != 12 || oi >= k.nObj) {
              atomicOr(a.iscal + IS_ERROR, ERR_TYPE);
              continue;
            }
            float* dst = gout + (size_t)(dj >> 8) * NP + x;
            const float gj = *dst;
            const float* ov = sObj + 6 * oi;
            const float wj = j <= 6 ? (float)WJ(1) : (float)WJ(7);
            const float cv = (mlk & OSTALE) ? 0.0f
                : __fmaf_rn((float)cx, ov[3], __fmaf_rn((float)cy, ov[4], (float)cz * ov[5]));
            const float BBi = 6.0f * s.n * wj * cv;
            const uint32_t so = a.solid[lk];
            if (so < (uint32_t)k.nObj) {
              if ((int)so != ocur) {
                if (ocur >= 0)
                  for (int c = 0; c < 6; ++c) atomicAdd(&accO[6 * ocur + c], fo[c]);
                for (int c = 0; c < 6; ++c) fo[c] = 0.0f;
                ocur = (int)so;
              }
              const float* os = sObj + 6 * so;
              const float bb = 2.0f * gj - BBi;
              const float Fx = (float)cx * bb, Fy = (float)cy * bb, Fz = (float)cz * bb;
              const float rx = (float)(ix + cx) - os[0];
              const float ry = (float)(iy + cy) - os[1];
              const float rz = (float)(iz + cz) - os[2];
              fo[0] += Fx;
              fo[1] += Fy;
              fo[2] += Fz;
              fo[3] += ry * Fz - rz * Fy;
              fo[4] += rz * Fx - rx * Fz;
              fo[5] += rx * Fy - ry * Fx;
            }
            *dst = gj - BBi;
            const double mo = t == 3 ? a.mass[x] : (double)a.nF[x];
            extra += (double)BBi * mo;
          }
          if (ocur >= 0)
            for (int c = 0; c < 6; ++c) atomicAdd(&accO[6 * ocur + c], fo[c]);
        }
      }
      if (act) {
        if (t == 3) {
          ++nif;
          appendInterface(x, a.ifList, a.iscal);
          a.rhoS[x] = s.n;
          a.uS[x] = s.ux;
          a.uS[NN + x] = s.uy;
          a.uS[2 * NN + x] = s.uz;
          a.hS[x] = s.hx;
          a.hS[NN + x] = s.hy;
          a.hS[2 * NN + x] = s.hz;
          atomicMin(&sbox[0], ix);
          atomicMin(&sbox[1], iy);
          atomicMin(&sbox[2], iz);
          atomicMax(&sbox[3], ix);
          atomicMax(&sbox[4], iy);
          atomicMax(&sbox[5], iz);
        } else if (k.freeSurface) {
          a.nF[x] = s.n;  // LB::updateMass fluid rule: mass = density
        }
      }
    }
    if (valid && nm != m) a.mask[x] = nm;
    if (useList) {  // keep this warp's activity bit of the chunk current
      const bool any = __any_sync(FULL, act);
      const unsigned bit = 1u << warp;
      const bool was = (sAct[sList[i]] & bit) != 0;
      if (lane == 0 && any != was) {
        if (any) atomicOr(k.chunkAct + c, bit);
        else atomicAnd(k.chunkAct + c, ~bit);
      }
    }
  }
  // no bulk copy may still be in flight when the block exits: on an early
  // exit, wait (bounded) for the copies issued beyond the last iteration used
#if LBDEM_MIXED_PRODUCER
  if (warp < MIXED_CONSUMERS / 32 && lane == 0) atomicMin(&sConsumed, i);
  __syncthreads();
  if (warp == MIXED_CONSUMERS / 32 && lane == 0)
    for (unsigned q = sConsumed; q < issued; ++q)
      if (!mbarWait(&fullBar[q % MIXED_STAGES], (q / MIXED_STAGES) & 1u))
        atomicOr(a.iscal + IS_ERROR, ERR_PIPELINE);
#else
  if (tid == 0)
    for (unsigned q = i; q < issued; ++q)
      if (!mbarWait(&fullBar[q % MIXED_STAGES], (q / MIXED_STAGES) & 1u))
        atomicOr(a.iscal + IS_ERROR, ERR_PIPELINE);
#endif
  // block totals
  nact = __reduce_add_sync(FULL, nact);
  nif = __reduce_add_sync(FULL, nif);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) extra += __shfl_xor_sync(FULL, extra, o);
  if (lane == 0) {
    if (nact) atomicAdd(&scnt[0], nact);
    if (nif) atomicAdd(&scnt[1], nif);
    if (extra != 0.0) atomicAdd(&accX, extra);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 6 * MAX_OBJ; i += blockDim.x) {
    if (accO[i] == 0.0f) continue;
    const int o = i / 6, c = i % 6;
    atomicAdd(a.obj + o * OB_STRIDE + (c < 3 ? OB_FHYDRO + c : OB_MHYDRO + c - 3),
              (double)accO[i]);
  }
  if (threadIdx.x == 0) {
    if (accX != 0.0) atomicAddComp(a.scal + SC_EXTRA_MASS, a.scal + SC_EXTRA_MASS_LO, accX);
    if (scnt[0]) atomicAdd(a.uscal + US_ACTIVE_UPDATES, (unsigned long long)scnt[0]);
    if (scnt[1]) atomicAdd(a.iscal + IS_NIF, (int)scnt[1]);
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

// Hydrodynamic force on the walls, mixed form: the wall branch of
// LB::streaming (src/LB.cpp:1334-1544) accumulates (2 (f_j - w_j rho0) - BBi) c_j
// with BBi = 0 for walls at rest, i.e. 2 g_j c_j in deviation form. For an
// active node x next to a wall node x + c_j, lbStepMixed stored g_j(x) in
// direction opp(j) of x (bounce-back), so the sums are formed here from the
// lattice it wrote, before anything else changes it. Walls are the outer
// node layer of the box (the only wall layout a run accepts), so only the
// layer inside it is visited, one face per blockIdx.y:
//   0, 1: x = 1, X-2 (all inner y, z)        2, 3: y = 1, Y-2 (x inside them)
//   4, 5: z = 1, Z-2 (x, y inside them)
// Each force goes to the wall that the wall node's solid index names, as in
// the reference: the wall setup gives a node on several faces the last of
// their walls in face order x0, x1, y0, y1, z0, z1, and the first flag reset
// (updateIndices) sets every wall node's index to 0 for good.
LBDEM_KERNEL(, lbWallForceMixed, LbArgs, lb) {
  __shared__ float accW[3 * MAX_WALL];
  for (int i = threadIdx.x; i < 3 * MAX_WALL; i += blockDim.x) accW[i] = 0.0f;
  __syncthreads();
  const int X = k.X, Y = k.Y, Z = k.Z;
  const int face = blockIdx.y, axis = face >> 1;
  // the face's node grid (u fastest, then v) and its fixed coordinate
  const int ux0 = axis == 0 ? 1 : 2, nu = axis == 0 ? Y - 2 : X - 4;
  const int vx0 = axis == 2 ? 2 : 1, nv = axis == 2 ? Y - 4 : Z - 2;
  const int fixed = (face & 1) ? (axis == 0 ? X : axis == 1 ? Y : Z) - 2 : 1;
  const bool reset = a.iscal[IS_WALLS_RESET] != 0;
  // a lattice 3 nodes wide has one inner layer: its second face is the first
  const bool dup = (face & 1) && fixed == 1;
  const float* gout = (const float*)a.fout;
  const size_t NP = (size_t)k.NP;
  float fw[3] = {0.0f, 0.0f, 0.0f};
  int wcur = -1;
  if (!dup && nu > 0 && nv > 0 && X > 2 && Y > 2 && Z > 2) {
    const unsigned total = (unsigned)nu * (unsigned)nv;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += gridDim.x * blockDim.x) {
      const int u = ux0 + (int)(t % (unsigned)nu), v = vx0 + (int)(t / (unsigned)nu);
      int ix, iy, iz;
      if (axis == 0) { ix = fixed; iy = u; iz = v; }
      else if (axis == 1) { ix = u; iy = fixed; iz = v; }
      else { ix = u; iy = v; iz = fixed; }
      const unsigned x = (unsigned)ix + (unsigned)iy * (unsigned)k.sy + (unsigned)iz * (unsigned)k.sz;
      if (!isActiveT(a.mask[x] & TYPE_MASK)) continue;
      const unsigned wl = boxWallLinks(k, ix, iy, iz);
#pragma unroll
      for (int j = 1; j < Q; ++j) {
        if (!((wl >> j) & 1u)) continue;
        const int tx = ix + CX(j), ty = iy + CY(j), tz = iz + CZ(j);
        const int w = reset ? 0
                    : tz == Z - 1 ? 5 : tz == 0 ? 4 : ty == Y - 1 ? 3 : ty == 0 ? 2
                    : tx == X - 1 ? 1 : 0;
        if (w >= k.nWall) continue;
        if (w != wcur) {
          if (wcur >= 0)
            for (int c = 0; c < 3; ++c) atomicAdd(&accW[3 * wcur + c], fw[c]);
          fw[0] = fw[1] = fw[2] = 0.0f;
          wcur = w;
        }
        const float bb = 2.0f * gout[OPPJ(j) * NP + x];
        if (CX(j)) fw[0] += CX(j) > 0 ? bb : -bb;
        if (CY(j)) fw[1] += CY(j) > 0 ? bb : -bb;
        if (CZ(j)) fw[2] += CZ(j) > 0 ? bb : -bb;
      }
    }
  }
  if (reset) {
    // one wall: a warp sum, then one shared atomic per component
    const unsigned FULLM = 0xffffffffu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      for (int c = 0; c < 3; ++c) fw[c] += __shfl_xor_sync(FULLM, fw[c], o);
    if ((threadIdx.x & 31) == 0 && k.nWall > 0)
      for (int c = 0; c < 3; ++c) atomicAdd(&accW[c], fw[c]);
  } else if (wcur >= 0) {
    for (int c = 0; c < 3; ++c) atomicAdd(&accW[3 * wcur + c], fw[c]);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * MAX_WALL; i += blockDim.x)
    if (accW[i] != 0.0f) atomicAdd(a.wallF + (i / 3) * 12 + (i % 3), (double)accW[i] * k.uForce);
}

}  // namespace lbdem
