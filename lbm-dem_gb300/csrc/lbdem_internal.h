// Internal definitions shared by the CUDA translation units of liblbdem.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <array>
#include <string>
#include <utility>
#include <vector>

#include "lbdem.h"

namespace lbdem {

constexpr int Q = 19;
constexpr int MAX_N = 50;        // neighbour-list slots, src/DEM.cpp:476
constexpr int MAX_L = 100000;    // cell-list cells,     src/DEM.cpp:479
constexpr int MAX_OBJ = 8;       // impactors handled on the device
constexpr int MAX_WALL = 6;
constexpr int MAX_BODY = 8;      // bodies (body.dat) handled on the device
constexpr int PAIR_VALS = 18;    // per neighbour slot: contact(6) lub(9) rep(3)
// per particle, mixed form: the 15 pair sums of the gather (FC, MC / radius,
// FL, ML, FR), padded to a 64-byte line
constexpr int SLOT_SUM_STRIDE = 16;
// steady cycles per replayed graph when no output file is open (even: the
// lattice buffers are back where they started)
#ifndef LBDEM_GRAPH_CYCLES
#define LBDEM_GRAPH_CYCLES 16
#endif
static_assert(LBDEM_GRAPH_CYCLES % 2 == 0, "an even number of cycles per graph");
#ifndef LBDEM_UNCOVER_CAP
#define LBDEM_UNCOVER_CAP 8192
#endif
constexpr int UNCOVER_CAP = LBDEM_UNCOVER_CAP;  // uncovered object nodes resolved per step
constexpr int ACCF_N = 13;       // mixed-form particle sums: d(3), r (x) d (9), mass(1)
constexpr int ACCF_STRIDE = 16;  // floats per particle: its sums share one 64-byte line

// mask byte layout
constexpr uint8_t TYPE_MASK = 0x0F;
constexpr uint8_t PFLAG = 0x10;   // inside a particle (nodeType::p)
constexpr uint8_t ABIT = 0x20;    // member of the last active list (cleanLists)
// Cache: every streaming neighbour was active, or a wall of the box's outer
// node layer, when the lattice step last checked. Set only by the lattice
// step; cleared around every node that leaves the active types
// (free-surface emptying, impactor voxelisation); box walls never change.
constexpr uint8_t BULK = 0x40;
// An impactor node outside every impactor, which only a restart file makes
// (its type comes from the file): in the reference it is in no object's
// node list, so it is never uncovered, and its node is recreated every
// step without the impactor's velocity (src/LB.cpp:822-839): links into it
// bounce back with zero wall velocity. Cleared when an impactor covers it.
constexpr uint8_t OSTALE = 0x80;

// device error bits
enum : int {
  ERR_TYPE = 1,          // streaming met a type the reference cannot stream to
  ERR_NBR_OVERFLOW = 2,  // > 49 neighbours
  ERR_CELL_OVERFLOW = 4, // > 50 particles in a cell or too many cells
  ERR_UNCOVER_CAP = 8,   // too many uncovered object nodes in one step
  ERR_PARTICLE_INDEX = 16,
  ERR_NONFINITE = 32,
  ERR_GRID = 64,         // particle outside the cell grid
  ERR_PIPELINE = 128,    // a bounded wait of the lattice step's copy pipeline gave up
};

// Physical / lattice constants of one run (passed by value to kernels).
struct Consts {
  int X, Y, Z;
  long long N;
  long long NP;      // population plane stride: N rounded up to a multiple of 256
  long long sy, sz;  // strides of y and z
  int freeSurface, forceField;
  double uLength, uTime, uSpeed, uAccel, uAngVel, uForce, uTorque, uVolume;
  double initDensity, initVisc;
  double omega, omegaf;  // 1/(0.5+3 visc), 1-1/(1+6 visc) (src/node.cpp:183,196)
  int mixed;             // FP32 deviation storage / FP32 collision form
  float omegaF, omegafF, lbFf[3];
  float sLF;             // unit.Length * unit.Force, stresslet scale (mixed form)
  float uForceF, uTorqueF, uVolumeF;  // the units in FP32 (mixed form)
  float invLengthF, invSpeedF, invAngVelF;  // their reciprocals (mixed form)
  // bound on |fl32(x0 / L) - x0 / L| in lattice units for positions in the
  // lattice, when formed as float(x0) * invLengthF
  float posErrF;
  double lbF[3];        // after the forceField reset rule of LB::collision
  double initVel[3];
  int nObj, nWall, nPart;
  // DEM
  double demSize[3];
  double dt;
  double k, c, mu, kinVisc, lubN, lubT, lubR, lubCut, electro, debye;
  int objWaitTime;
  // mixed form: per 256-node chunk, bit w set = warp w of the chunk may hold
  // active nodes (the lattice step skips chunks with no bit set); null in
  // the plain form
  uint32_t* chunkAct;
  // per direction j: neighbour offset cx + cy sy + cz sz, and the push
  // target of population j relative to a node, j NP + that offset (both in
  // elements; 19 NP < 2^32 is checked when the run is created)
  int nbOff[Q];
  unsigned pushOff[Q];
  int debugFlags;  // lbdem_options::debug_flags (failure-path tests only)
  // rheology (plain form): model, parameters in lattice units, and the
  // per-node viscosity (null for a Newtonian run without turbulence, whose
  // every node has initVisc)
  int rheo, turbulence;
  double plasticVisc, yieldStress, frictionCoef, voellmyCoef, turbConst;
  double* visc;
  // bodies and their springs to the impactors (DEM::bodyObjectInteraction)
  int nBody, nonLinType;
  double springDamp, k13, epsilon;
  // the type of every wall node (5-8) and the slip coefficient S1 = slip,
  // S2 = 1 - slip of slip walls (LB::streaming, src/LB.cpp:1337-1352)
  int wallType;
  double slipS1, slipS2;
  float slipS1f, slipS2f;
};

struct DeviceWall {
  double p[3], n[3];
};

// All device allocations of one run.
struct Device {
  // lattice
  uint8_t* mask = nullptr;
  uint32_t* solid = nullptr;
  uint8_t* objIdx = nullptr;   // object whose velocity an object node carries
  uint32_t* claim = nullptr;   // particle claims during updateIndices
  uint8_t* fsflag = nullptr;   // transient free-surface flags
  void* f[2] = {nullptr, nullptr};  // distributions, ping-pong
  double* mass = nullptr;
  float* nF = nullptr;         // fluid-node density, mixed form only
  double* massNew = nullptr;
  double* visc = nullptr;      // per-node viscosity (rheology runs only)
  double* rhoS = nullptr;      // density of interface nodes
  double* uS = nullptr;        // shifted velocity of interface nodes [3][N]
  double* hS = nullptr;        // hydrodynamic force of interface nodes [3][N]
  // scalars / reductions (double unless noted)
  double* scal = nullptr;      // see SC_* offsets
  int* iscal = nullptr;        // see IS_* offsets
  unsigned long long* uscal = nullptr;
  // particles (SoA, [3][P] for vectors)
  double *px0 = nullptr, *px1 = nullptr, *pw1 = nullptr;
  double *pr = nullptr, *pinvm = nullptr, *pinvI = nullptr;
  double *pFHydro = nullptr, *pMHydro = nullptr, *pFluidVol = nullptr, *pSHydro = nullptr;
  double *pFContact = nullptr, *pMContact = nullptr, *pFLub = nullptr, *pMLub = nullptr;
  double *pFRep = nullptr, *pFTotal = nullptr, *pMTotal = nullptr, *pFGrav = nullptr;
  double *pxiw = nullptr, *pxio = nullptr;
  double* pkd = nullptr;                 // [6][P] lattice-unit kinematics
  float* pkf = nullptr;                  // [P][12] float4 x0/L, x1/S, w1/W (mixed form)
  float* pAccF = nullptr;                // [P][ACCF_STRIDE] particle sums (mixed form)
  uint32_t* chunkAct = nullptr;          // [NP/256] chunk activity (mixed form)
  int* plist[2] = {nullptr, nullptr};    // [P][50]
  double* pxi[2] = {nullptr, nullptr};   // [P][3][50]
  int* partner = nullptr;                // [P][50] slot of i in list[j]
  int* gorder = nullptr;                 // [P][50] gather order of slots
  int* pairList = nullptr;               // [25 P] owner slots i*50+s with list[i][s] < i
  double* pairbuf = nullptr;             // [P][50][PAIR_VALS]
  uint8_t* pairflag = nullptr;           // [P][50] bit0 = lubrication valid
  float* slotSum = nullptr;              // [P][SLOT_SUM_STRIDE] mixed form
  int* pcell = nullptr;                  // [P] cell of particle
  float4* posf = nullptr;                // [P] FP32 position and radius (list rebuilds)
  float4* kinf = nullptr;                // [P][2] mixed form: (v, r), (w, 0) in FP32
  int* ppos = nullptr;                   // [P] position in its cell (1-based)
  int* cellCount = nullptr;              // [MAX_L]
  int* cellStart = nullptr;              // [MAX_L]
  int* cellFill = nullptr;               // [MAX_L]
  int* cellParts = nullptr;              // [P]
  // objects / walls (small)
  double* obj = nullptr;                 // see OB_* layout, [nObj][OB_STRIDE]
  double* body = nullptr;                // see BD_* layout, [nBody][BD_STRIDE]
  double* wallF = nullptr;               // [W][12]: FHydro FContact FLub FTotal
  DeviceWall* walls = nullptr;
  uint32_t* uncover = nullptr;           // [UNCOVER_CAP] candidate list
  uint32_t* ifList = nullptr;            // [N] interface nodes of the lattice step, any order
  double* stress = nullptr;              // [36] DEM stress sums of an output cycle (demStress)
  double* pStress = nullptr;             // [9][P] per-particle total stresslet (same cycles)
  double* xinitY = nullptr;              // [P] particle::x_i.y
  double* dispY = nullptr;               // [P] particle::disp.y
};

// offsets into Device::scal (doubles)
enum {
  SC_EXTRA_MASS = 0,  // bounce-back extra mass of this LB step
  SC_ADD_MASS,        // extraMass / #interface
  SC_SURPLUS,         // free-surface mass surplus
  SC_MAXDISP,         // DEM::maxDisp
  SC_TOTAL_MASS,      // diagnostics
  // compensation terms of the two mass-budget sums: the rounding error of
  // every atomic addition to SC_EXTRA_MASS / SC_SURPLUS (atomicAddComp)
  SC_EXTRA_MASS_LO,
  SC_SURPLUS_LO,
  SC_COUNT
};
// offsets into Device::iscal (ints)
enum {
  IS_ERROR = 0,
  IS_NEWNBR,        // DEM::newNeighborList
  IS_REBUILD,       // neighbour list rebuild requested in this DEM step
  IS_NIF,           // interface count after the LB step (redistribution)
  IS_NIF2,          // interface count after removeIsolated
  IS_BBOX,          // 6 ints: xmin,ymin,zmin,xmax,ymax,zmax of interface nodes
  IS_NUNCOVER = IS_BBOX + 6,
  IS_NL = IS_NUNCOVER + 1,  // 3 ints: nlx, nly, nlz
  IS_DIRECT = IS_NL + 3,    // direct-sum branch in use
  IS_LISTCUR,               // which list buffer is current
  IS_REBUILDS,              // rebuild counter
  IS_NPAIRS,                // entries of the owner-pair list
  IS_BLOCKS_DONE,           // demBegin: blocks that have posted their maximum
  IS_DEMSTEP,               // DEM::demTimeStep, advanced by demBegin
  IS_GATHER_DONE,           // demGather: blocks done (the last one updates the impactors)
  IS_PAIRLIST_DONE,         // nbrPairList: blocks done (the last one swaps the lists)
  IS_WALLS_RESET,           // set by the first flag reset: every wall node has solid index 0
  IS_IFLIST,                // entries of Device::ifList written by this lattice step
  IS_COUNT
};
// offsets into Device::uscal
enum { US_FIRSTFLAG = 0, US_ACTIVE_UPDATES,
       US_MAXV2,  // demBegin: max |x1|^2 as the bit pattern of a non-negative double
       US_COUNT };

// object record layout (doubles)
enum {
  OB_X0 = 0, OB_X1 = 3, OB_W1 = 6, OB_R = 9, OB_INVM = 10, OB_INVI = 11,
  OB_FHYDRO = 12, OB_MHYDRO = 15, OB_FCONTACT = 18, OB_MCONTACT = 21,
  OB_FLUB = 24, OB_MLUB = 27, OB_FGRAV = 30, OB_FTOTAL = 33, OB_MTOTAL = 36,
  OB_X0PREV = 39, OB_INDEX = 42,
  OB_MASS = 44,     // object::m (the body springs' damping)
  OB_FSPRING = 45,  // object::FSpring, set by the body springs
  OB_STRIDE = 48
};

// body record layout (doubles), src/elmt.h:231-258
enum {
  BD_X0 = 0, BD_X1 = 3, BD_R = 6, BD_M = 7, BD_INVM = 8, BD_K = 9, BD_L0 = 10, BD_L = 11,
  BD_FGRAV = 12, BD_FSPRING = 15, BD_FTOTAL = 18, BD_STRIDE = 24
};

}  // namespace lbdem

namespace lbdem {
struct JobArgs;
}
struct lbdem_output;  // screen-phase output files (output.cu)
// after each goCycle of lbdem_cycle: advance the output clock one cycle and
// enqueue the copy of the state if a line is due
int lbdemOutputAfterCycle(lbdem_ctx* c);
// lbdem_create under lbRestart: types and fields from the fluid recycle file
int lbdemRestartFluid(lbdem_ctx* c, const char* path);
// whether the next cycle is an output cycle
bool lbdemOutputDueNext(const lbdem_ctx* c);
// whether the next cycle's DEM step forms the stress sums (a stress-file line
// follows it)
bool lbdemOutputStressNext(const lbdem_ctx* c);
// whether it also forms the per-particle totals (a particle recycle file
// follows it)
bool lbdemOutputParticleStressNext(const lbdem_ctx* c);
// whether two cycles cannot run as one replayed pair: an output is due after
// the first, or the stress sums are due in the second
bool lbdemOutputBlocksPair(const lbdem_ctx* c);
// write the lines whose copies have completed (all of them, waiting, if wait)
int lbdemOutputDrain(lbdem_ctx* c, bool wait);
void lbdemOutputFree(lbdem_ctx* c);
// after a restore: the output clock of the restored cycle count (pending
// lines are written first; no line for the current cycle)
void lbdemOutputResync(lbdem_ctx* c);
extern "C" int lbdem_export_recycle_fluid(lbdem_ctx* c, const char* path);
// many runs per launch (lbdem_capi.cu), for the run server
void lbdemJobArgs(lbdem_ctx* c, int cur, lbdem::JobArgs* j);
bool lbdemBatchable(const lbdem_ctx* c);
int lbdemBatchKey(const lbdem_ctx* c);
int lbdemEnqueueBatchCycle(const std::vector<lbdem_ctx*>& runs, const lbdem::JobArgs* jobs,
                           cudaStream_t s);
void lbdemAdvanceCounters(lbdem_ctx* c, int cycles);
// Enqueues on stream st a check that the run's particle and impactor
// positions, velocities and hydrodynamic forces and its interface mass share
// are finite (ERR_NONFINITE otherwise), then a copy
// of its device error bits into dst (pinned host memory), for a check once
// st reaches that point.
int lbdemEnqueueErrorRead(lbdem_ctx* c, int* dst, cudaStream_t st);
// The status of error bits read that way (LBDEM_OK for 0); sets the run's
// message.
int lbdemErrorStatus(lbdem_ctx* c, int bits, const char* when);

// Counts one device allocation for lbdem_device_allocations; every
// cudaMalloc / cudaMallocAsync of the library calls it.
void lbdemNoteDeviceAllocation();

// Makes a device current for the length of one entry point and puts the
// calling thread's previous device back on exit, so that contexts on
// different devices can be driven from one host thread.
struct DeviceScope {
  int prev = -1;
  int dev;
  explicit DeviceScope(int d) : dev(d) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      prev = -1;
      return;
    }
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceScope() {
    if (prev >= 0 && prev != dev) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

struct lbdem_ctx {
  std::string err;
  lbdem::Consts k{};
  lbdem::Device d;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  // mixed form, captured cycles: the free-surface step of a cycle runs on
  // fsStream beside the next cycle's DEM step (fsFork / fsDone order it)
  cudaStream_t fsStream = nullptr;
  cudaEvent_t fsFork = nullptr, fsDone = nullptr;
  bool fsPending = false;  // a forked free-surface step not yet joined
  bool directList = false;  // DEM neighbour list by direct sums (fixed at creation)
  // mixed form, captured cycles: lbPrepare runs on sideStream beside the
  // coupling step, and the wall-force sweep beside the finalisation and the
  // interface mass update (joined before the interface types change) and
  // the next DEM step (joined before the gather, which reads the wall sums)
  bool overlap = false;
  cudaStream_t sideStream = nullptr;
  cudaEvent_t prepFork = nullptr, prepDone = nullptr, wallFork = nullptr, wallDone = nullptr;
  bool prepPending = false, wallPendingFs = false, wallPendingMain = false;
  // the next cycle's DEM step up to its gather, on demStream beside this
  // cycle's lattice and free-surface steps (joined before that gather)
  cudaStream_t demStream = nullptr;
  cudaEvent_t demFork = nullptr, demDone = nullptr;
  bool demPrePending = false;
  int device = 0;
  int precision = LBDEM_PLAIN_FP64;
  int check_every = 0;
  int cur = 0;  // current lattice buffer
  // host-side mirrors of the reference's step counters
  bool demSolve = false, lbSolve = false, freeSurface = false;
  double demInitialRepeat = 0.0;
  double demTime = 0.0;
  long long demTimeStep = 0, lbTime = 0;
  bool lbFReset = false;  // lbF reset by the first collision when !forceField
  double lbFConfig[3] = {0, 0, 0};
  int nPart = 0, nObj = 0, nWall = 0, nBody = 0;
  double fluidHeight = 0.0;     // physical, as the configuration gives it
  lbdem_output* out = nullptr;  // open screen-phase output files, if any
  bool stressNext = false;      // the next DEM step forms the stress sums
  bool pStressNext = false;     // ... and the per-particle totals
  int objIndexField[lbdem::MAX_OBJ] = {0};
  long long deviceBytes = 0;
  // every device allocation of the run, in allocation order (the same order
  // and sizes for every run created from one configuration and form): what
  // a snapshot holds, and what lbdem_destroy frees
  std::vector<std::pair<void*, size_t>> buffers;
  int smCount = 0;
  int lbMixedBlocks = 0;  // resident blocks of the mixed lattice kernel (one wave)
  int chunksPerBlock = 8; // at least this many 256-node chunks per lattice block
  int gridLattice = 1;    // mixed lattice grid: one wave, or fewer for a small run
  // grids of the per-cycle kernels, sized by their work (fixed per run):
  // the free-surface area, the wall-adjacent layer, the impactor boxes and
  // the neighbour cells; grid-stride loops cover any excess
  int gridFs = 1, gridShell = 1, gridObj = 1, gridCells = 1;
  // measurement
  bool profiling = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> lbEvents;
  size_t lbEventsUsed = 0;
  // per profiled cycle: events before the DEM step and after each of the
  // four steps
  std::vector<std::array<cudaEvent_t, 5>> phaseEvents;
  size_t phaseEventsUsed = 0;
  long long launches = 0;
  // two goCycles as one CUDA graph, per starting lattice buffer
  cudaGraphExec_t pairGraph[2] = {nullptr, nullptr};
  cudaGraphExec_t oneGraph[2] = {nullptr, nullptr};  // single cycles, per start buffer
  // groups of steady cycles when no output is open: [0] 4 cycles, [1]
  // LBDEM_GRAPH_CYCLES cycles (calls of many cycles), per start buffer
  cudaGraphExec_t groupGraph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  long long groupKernels[2] = {0, 0};
  long long oneKernels = 0;
  long long pairKernels = 0;
};
