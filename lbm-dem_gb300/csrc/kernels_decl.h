// Kernel argument blocks and kernel prototypes shared by the host sequencing
// (lbdem_capi.cu) and the kernel translation units.
#pragma once
#include "lbdem_internal.h"

namespace lbdem {

struct LbArgs {
  const void* fin;    // double (plain) or float deviations f - w (mixed)
  void* fout;
  float* nF;          // density of fluid nodes (mixed form)
  uint8_t* mask;
  const uint32_t* solid;
  const uint8_t* objIdx;
  double* mass;
  double* rhoS;
  double* uS;
  double* hS;
  const double* px0;
  const double* px1;
  const double* pw1;
  const double* pkd;  // [6][P] x0/L, x1/S (double)
  const float* pkf;   // [P][12]: float4 x0/L, x1/S, w1/W (mixed form)
  double* pFHydro;    // [3][P] lattice-unit sums
  double* pMHydro;    // [3][P]
  double* pSHydro;    // [9][P]
  double* pFluidVol;  // [P]
  float* pAccF;       // [P][ACCF_STRIDE] float particle sums (mixed form)
  double* obj;        // object records
  double* wallF;      // [W][12]
  double* scal;
  int* iscal;
  unsigned long long* uscal;
  uint32_t* ifList;   // interface nodes of this step, appended (IS_IFLIST entries)
};

struct FsArgs {
  void* fcur;          // post-stream populations (current lattice)
  const void* fold;    // pre-collision populations of this step
  float* nF;           // density of fluid nodes (mixed form)
  uint8_t* mask;
  const uint32_t* solid;
  const uint8_t* objIdx;
  uint8_t* fsflag;
  double* mass;
  double* massNew;
  double* rhoS;
  const double* uS;
  const double* hS;
  const double* px0;
  const double* px1;
  const double* pw1;
  const double* pkd;
  const float* pkf;
  const double* obj;
  double* scal;
  int* iscal;
  const uint32_t* ifList;  // interface nodes after the lattice step (IS_IFLIST entries)
};

struct DemArgs {
  double *x0, *x1, *w1, *r, *invm, *invI;
  double *FHydro, *MHydro, *FContact, *MContact, *FLub, *MLub, *FRep, *FTotal, *MTotal,
      *FGrav;
  double *xiw, *xio;
  int* list[2];
  double* xi[2];
  int* partner;
  int* gorder;
  int* pairList;
  double* pairbuf;
  uint8_t* pairflag;
  float* slotSum;  // [P][SLOT_SUM_STRIDE] mixed form: demSlotSumsMixed -> demGatherMixed
  int* pcell;
  float4* posf;  // [P] FP32 position and radius, written by nbrCellAssign
  float4* kinf;  // [P][2] mixed form: (v, r) and (w, 0) in FP32, written by demBegin
  // particle::x_i.y (position at the start, again after the objWaitTime
  // step) and disp.y = x_i.y - x0.y after each integration (src/DEM.cpp:288,
  // 2705, 2721-2724); read only by the particle recycle file
  double* xinitY;
  double* dispY;
  int* ppos;
  int *cellCount, *cellStart, *cellFill, *cellParts;
  double* obj;
  double* wallF;
  const DeviceWall* walls;
  double* scal;
  int* iscal;
  unsigned long long* uscal;
  double* body;
};

// Pointers of one run's coupling kernels (impactor uncover and voxelisation,
// particle flags), of the lattice step's preparation and finalisation.
struct CoupArgs {
  uint8_t* mask;
  uint32_t* solid;
  uint8_t* objIdx;
  uint32_t* claim;
  double* mass;
  float* nF;
  void* fcur;  // current lattice (uncovered nodes are initialised in it)
  uint32_t* uncover;
  double *px0, *px1, *pw1, *pr;
  double* obj;
  double* wallF;
  double* scal;
  int* iscal;
  unsigned long long* uscal;
  double* pAcc;  // hydrodynamic accumulators, reset by lbPrepare
  long long pAccLen;
  float* pAccF;
  long long pAccFLen;
  double* pkd;
  float* pkf;
  double *pF, *pM, *pV, *pS;  // particle force, torque, volume, stresslet
  int redistribute;           // free surface on: mass redistribution
};

// Everything the per-cycle kernels of one run take. Launches that advance
// many runs at once (blockIdx.z = run) read one record per run; a run has one
// record per cycle parity (the lattice buffers swap every cycle).
struct JobArgs {
  Consts k;
  DemArgs dem;
  LbArgs lb;
  FsArgs fs;
  CoupArgs cp;
};

// Copy a record into shared memory; every thread of the block takes part,
// and a __syncthreads() must follow before it is read.
template <class T>
__device__ __forceinline__ void stageRecord(T& dst, const T& src) {
  static_assert(sizeof(T) % 8 == 0, "records are 8-byte multiples");
  const unsigned long long* s = reinterpret_cast<const unsigned long long*>(&src);
  unsigned long long* d = reinterpret_cast<unsigned long long*>(&dst);
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 8); i += blockDim.x) d[i] = s[i];
}

// Parameters of the single-run entry points: grid constants, so that
// passing them on by reference (to functions that are not inlined) reads
// the parameter space instead of copying the records to local memory.
#define LBDEM_KPARAMS(ARGT) const __grid_constant__ Consts k, const __grid_constant__ ARGT a

// A kernel taking (Consts, ARGT) in two entry points: NAME for one run
// (arguments by value) and NAME##Batch for many runs at once, which stages
// run blockIdx.z's record in shared memory. Both run NAME##Body, which
// follows the macro as the function body.
#define LBDEM_KERNEL(BOUNDS, NAME, ARGT, FIELD)                                  \
  __device__ __forceinline__ void NAME##Body(const Consts& k, const ARGT& a);   \
  __global__ void BOUNDS NAME(LBDEM_KPARAMS(ARGT)) { NAME##Body(k, a); }       \
  __global__ void BOUNDS NAME##Batch(const JobArgs* jobs) {                     \
    __shared__ __align__(16) Consts sk;                                          \
    __shared__ __align__(16) ARGT sa;                                            \
    stageRecord(sk, jobs[blockIdx.z].k);                                         \
    stageRecord(sa, jobs[blockIdx.z].FIELD);                                     \
    __syncthreads();                                                             \
    NAME##Body(sk, sa);                                                          \
  }                                                                              \
  __device__ __forceinline__ void NAME##Body(const Consts& k, const ARGT& a)

// Mixed lattice step launch shape: chunks of MIXED_CHUNK consecutive nodes
// (one consumer thread per node), staged through MIXED_STAGES shared-memory
// buffers of 19 FP32 planes, the solid indices, the fluid densities nF and
// the mask bytes, which a producer warp of each block fills with bulk
// copies. Measured on GB300 (256x320x256 lattice, 15.4 M active nodes):
//   producer warp, 2 blocks/SM, 3 stages      0.507 ms  (the default)
//   thread 0 of warp 0 issuing, 3 blocks/SM   0.543 ms
//   thread 0 issuing, 2 blocks/SM             0.686 ms
//   producer, 3 blocks/SM                     0.538 ms
//   producer, 2 blocks/SM, 2 or 4 stages      0.509-0.510 ms
//   solid indices and nF read from global memory by particle nodes instead of
//   staged: 0.579 ms at 2 blocks/SM, 0.509 ms at 3
// The knobs stay compile-time options (-D) for re-measurement.
constexpr int MIXED_CHUNK = 256;
#ifndef LBDEM_MIXED_STAGES
#define LBDEM_MIXED_STAGES 3
#endif
#ifndef LBDEM_MIXED_MIN_BLOCKS
#define LBDEM_MIXED_MIN_BLOCKS 2
#endif
// resident lattice blocks per SM at most (the grid is one resident wave)
#ifndef LBDEM_MIXED_MAX_PER_SM
#define LBDEM_MIXED_MAX_PER_SM 2
#endif
constexpr int MIXED_STAGES = LBDEM_MIXED_STAGES;
// LBDEM_MIXED_STAGE_SIDE 1: the solid indices and fluid densities of a chunk
// are staged with its populations; 0: particle nodes (the only readers) load
// theirs from global memory, and a stage holds the populations and mask bytes
#ifndef LBDEM_MIXED_STAGE_SIDE
#define LBDEM_MIXED_STAGE_SIDE 1
#endif
constexpr int MIXED_STAGE_SOLID = Q * MIXED_CHUNK * 4;                 // byte offsets
constexpr int MIXED_STAGE_NF = MIXED_STAGE_SOLID + MIXED_CHUNK * 4;
constexpr int MIXED_STAGE_MASK =
    LBDEM_MIXED_STAGE_SIDE ? MIXED_STAGE_NF + MIXED_CHUNK * 4 : Q * MIXED_CHUNK * 4;
constexpr int MIXED_STAGE_BYTES = MIXED_STAGE_MASK + MIXED_CHUNK;
// LBDEM_MIXED_PRODUCER 1: an extra warp of each block issues the bulk copies
// (iteration q once every consumer warp has released iteration
// q - MIXED_STAGES); 0: thread 0 issues them between its own nodes
#ifndef LBDEM_MIXED_PRODUCER
#define LBDEM_MIXED_PRODUCER 1
#endif
constexpr int MIXED_CONSUMERS = MIXED_CHUNK;
constexpr int MIXED_THREADS = MIXED_CONSUMERS + 32 * LBDEM_MIXED_PRODUCER;
constexpr int MIXED_SMEM = MIXED_STAGES * MIXED_STAGE_BYTES;
#define MIXED_BOUNDS __launch_bounds__(MIXED_THREADS, LBDEM_MIXED_MIN_BLOCKS)
// chunks per block up to which inactive chunks are skipped (per-block list)
constexpr int MIXED_MAX_MINE = 2048;

// lb_fp64.cu / lb_mixed.cu
__global__ void lbStepFp64(LBDEM_KPARAMS(LbArgs));
__global__ void lbStepFp64Batch(const JobArgs* jobs);
__global__ void lbStepFp64Rheo(LBDEM_KPARAMS(LbArgs));
__global__ void lbStepFp64RheoBatch(const JobArgs* jobs);
__global__ void lbStepMixed(LBDEM_KPARAMS(LbArgs));
__global__ void lbStepMixedBatch(const JobArgs* jobs);
__global__ void lbWallForceMixed(LBDEM_KPARAMS(LbArgs));
__global__ void lbWallForceMixedBatch(const JobArgs* jobs);
__global__ void lbPrepare(Consts k, double* pAcc, long long pAccLen, float* pAccF,
                          long long pAccFLen, double* obj, double* wallF, double* scal,
                          int* iscal, const double* px0, const double* px1, const double* pw1,
                          double* pkd, float* pkf);
__global__ void lbFinalizeKernel(Consts k, double* pF, double* pM, double* pV, double* obj,
                                 double* wallF, double* scal, const int* iscal,
                                 const float* pAccF, double* pS, FsArgs fa, int redistribute);
__global__ void fsUpdateMass(LBDEM_KPARAMS(FsArgs));
__global__ void fsUpdateMassBatch(const JobArgs* jobs);
__global__ void fsMutants(LBDEM_KPARAMS(FsArgs));
__global__ void fsMutantsBatch(const JobArgs* jobs);
__global__ void fsSmoothen(LBDEM_KPARAMS(FsArgs));
__global__ void fsSmoothenBatch(const JobArgs* jobs);
__global__ void fsMutantsAndFill(LBDEM_KPARAMS(FsArgs));
__global__ void fsMutantsAndFillBatch(const JobArgs* jobs);
__global__ void fsEmptyIsolated(LBDEM_KPARAMS(FsArgs));
__global__ void fsEmptyIsolatedBatch(const JobArgs* jobs);
__global__ void fsRedistribute(LBDEM_KPARAMS(FsArgs));
__global__ void fsRedistributeBatch(const JobArgs* jobs);
__global__ void uncoverCollect(Consts k, const uint8_t* mask, const uint32_t* solid,
                               const double* obj,
                               uint32_t* list, int* iscal);
// dynamic shared memory of uncoverResolve: candidates, their lower-index
// candidate neighbours and states
constexpr int UNCOVER_SMEM = UNCOVER_CAP * (4 + 9 * 2 + 1);
// uncovered nodes up to this many are resolved by one thread in order
constexpr int UNCOVER_SERIAL = 256;
__global__ void uncoverResolve(Consts k, uint8_t* mask, void* f, double* mass, float* nF,
                               uint32_t* list, int* iscal);
__global__ void voxelizeObjects(Consts k, uint8_t* mask, uint32_t* solid, uint8_t* objIdx,
                                double* mass, double* obj);
__global__ void flagClaim(Consts k, const uint8_t* mask, uint32_t* claim, const double* px0,
                          const double* pr, const int* iscal, unsigned long long* uscal);
__global__ void flagApply(Consts k, uint8_t* mask, uint32_t* solid, uint32_t* claim,
                          int* iscal, unsigned long long* uscal);
__global__ void findNewActiveKernel(Consts k, uint8_t* mask, uint32_t* solid,
                                    const double* px0, const double* pr, int* iscal,
                                    unsigned long long* uscal);
__global__ void initTypes(Consts k, uint8_t* mask, uint32_t* solid, uint8_t* objIdx,
                          const int* boundary, const DeviceWall* walls, const int* wallType,
                          const double* obj, double fluidHeightLattice, int freeSurface);
__global__ void fillDouble(double* v, long long n, double value);
__global__ void slipStash(Consts k, const uint8_t* mask, void* f);
__global__ void slipApply(Consts k, const uint8_t* mask, void* f);
__global__ void initFields(Consts k, uint8_t* mask, void* f, double* mass, float* nF,
                           double fluidHeightLattice, int freeSurface);
// mass of the active nodes (outside particles unless withParticles), counts
__global__ void massSummaryKernel(Consts k, const uint8_t* mask, const double* mass,
                                  const float* nF, double* out, unsigned long long* cnt,
                                  int withParticles);
__global__ void momentsKernel(Consts k, const uint8_t* mask, const void* f, double* n,
                              double* u);
__global__ void nonfiniteCheck(Consts k, const uint8_t* mask, const void* f, int* iscal);
__global__ void motionFiniteCheck(const double* px0, const double* px1, const double* pFH,
                                  int n3, const double* obj, int nObj, const double* scal,
                                  int* iscal);
__global__ void exportLattice(Consts k, const uint8_t* mask, const void* f, const double* mass,
                              const float* nF, double* fOut, double* massOut);

// threads per block of the gather pass (one thread per particle): small
// blocks spread a few thousand particles over every SM
constexpr int GATHER_THREADS = 64;
// mixed-form pair sums (demSlotSumsMixed): GATHER_MIXED_LANES lanes per
// particle split its neighbour slots (the slot loop is a chain of dependent
// loads), so a block of GATHER_MIXED_THREADS holds GATHER_MIXED_PARTS
// particles
#ifndef LBDEM_GATHER_LANES
#define LBDEM_GATHER_LANES 8
#endif
constexpr int GATHER_MIXED_LANES = LBDEM_GATHER_LANES;
constexpr int GATHER_MIXED_THREADS = 128;
constexpr int GATHER_MIXED_PARTS = GATHER_MIXED_THREADS / GATHER_MIXED_LANES;
// DEM stress sums: contact, lubrication, electrostatic, hydrodynamic (3x3 each)
constexpr int STRESS_N = 36;
__global__ void demStress(Consts k, DemArgs a, const double* SHydro, double* out,
                          double* perParticle);

// dem_fp64.cu
__global__ void demBegin(Consts k, DemArgs a, int forceRebuild);
__global__ void nbrCellAssign(LBDEM_KPARAMS(DemArgs));
__global__ void nbrCellAssignBatch(const JobArgs* jobs);
__global__ void nbrCellScan(LBDEM_KPARAMS(DemArgs));
__global__ void nbrCellScanBatch(const JobArgs* jobs);
__global__ void nbrCellScatter(LBDEM_KPARAMS(DemArgs));
__global__ void nbrCellScatterBatch(const JobArgs* jobs);
__global__ void nbrCellSort(LBDEM_KPARAMS(DemArgs));
__global__ void nbrCellSortBatch(const JobArgs* jobs);
__global__ void nbrBuildCells(LBDEM_KPARAMS(DemArgs));
__global__ void nbrBuildCellsBatch(const JobArgs* jobs);
__global__ void nbrBuildDirect(LBDEM_KPARAMS(DemArgs));
__global__ void nbrBuildDirectBatch(const JobArgs* jobs);
__global__ void nbrDirectHistory(LBDEM_KPARAMS(DemArgs));
__global__ void nbrDirectHistoryBatch(const JobArgs* jobs);
__global__ void nbrPartners(LBDEM_KPARAMS(DemArgs));
__global__ void nbrPartnersBatch(const JobArgs* jobs);
__global__ void nbrPairList(LBDEM_KPARAMS(DemArgs));
__global__ void nbrPairListBatch(const JobArgs* jobs);
// the DEM step number comes from iscal[IS_DEMSTEP] (advanced by demBegin)
__global__ void demPairs(LBDEM_KPARAMS(DemArgs));
__global__ void demPairsBatch(const JobArgs* jobs);
__global__ void demGather(LBDEM_KPARAMS(DemArgs));
__global__ void demGatherBatch(const JobArgs* jobs);
// dem_mixed.cu: the force passes of the mixed form (FP32 force laws)
__global__ void demPairsMixed(LBDEM_KPARAMS(DemArgs));
__global__ void demPairsMixedBatch(const JobArgs* jobs);
__global__ void demSlotSumsMixed(LBDEM_KPARAMS(DemArgs));
__global__ void demSlotSumsMixedBatch(const JobArgs* jobs);
__global__ void demGatherMixed(LBDEM_KPARAMS(DemArgs));
__global__ void demGatherMixedBatch(const JobArgs* jobs);

// many-run entry points of the kernels with their own parameter lists
__global__ void demBeginBatch(const JobArgs* jobs);
__global__ void lbPrepareBatch(const JobArgs* jobs);
__global__ void lbFinalizeKernelBatch(const JobArgs* jobs);
__global__ void uncoverCollectBatch(const JobArgs* jobs);
__global__ void uncoverResolveBatch(const JobArgs* jobs);
__global__ void voxelizeObjectsBatch(const JobArgs* jobs);
__global__ void flagClaimBatch(const JobArgs* jobs);
__global__ void flagApplyBatch(const JobArgs* jobs);
__global__ void findNewActiveKernelBatch(const JobArgs* jobs);

}  // namespace lbdem
