// C ABI of liblbdem: context lifecycle, the step entry points and state
// download. The host side only sequences kernels on the context's stream;
// every step entry point enqueues work and returns without synchronising.
//
// Host arithmetic that feeds the kernels (units, masses, damping) follows
// the reference operation by operation (src/node.cpp:512-525,
// src/LB.cpp:153-330, src/DEM.cpp:199-357, src/elmt.cpp:27-63) and is
// compiled without FMA contraction, so device and reference start from the
// same bits.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbdem_internal.h"

#include "kernels_decl.h"
#include "lattice_common.cuh"

using namespace lbdem;

namespace {

const double PI_D = 3.14159265358979323846;

int setErr(lbdem_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess)                                                        \
      return setErr(ctx, _e == cudaErrorMemoryAllocation ? LBDEM_ERR_OOM : LBDEM_ERR_CUDA, \
                    std::string(#call) + ": " + cudaGetErrorString(_e));         \
  } while (0)

// Context memory comes from the stream-ordered allocator on the context's
// own stream: freeing it (lbdem_destroy) then waits for that stream only,
// not for the whole device, so runs sharing a GPU do not stall each other.
template <class T>
int dalloc(lbdem_ctx* ctx, T** p, size_t count) {
  const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  lbdemNoteDeviceAllocation();
  cudaError_t e = cudaMallocAsync((void**)p, bytes, ctx->stream);
  if (e != cudaSuccess)
    return setErr(ctx, LBDEM_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
  ctx->deviceBytes += (long long)bytes;
  ctx->buffers.emplace_back((void*)*p, bytes);
  cudaMemsetAsync(*p, 0, bytes, ctx->stream);
  return LBDEM_OK;
}

// frees a buffer taken with dalloc that the run does not keep
void dfree(lbdem_ctx* ctx, void* p) {
  for (size_t i = 0; i < ctx->buffers.size(); ++i)
    if (ctx->buffers[i].first == p) {
      ctx->deviceBytes -= (long long)ctx->buffers[i].second;
      ctx->buffers.erase(ctx->buffers.begin() + (long)i);
      break;
    }
  cudaFreeAsync(p, ctx->stream);
}

int launchErr(lbdem_ctx* ctx, const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return setErr(ctx, LBDEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return LBDEM_OK;
}

int latticeGrid(lbdem_ctx* ctx) { return std::max(1, ctx->smCount) * 8; }

// The status of a run's device error bits (0: LBDEM_OK), with a message.
int deviceError(lbdem_ctx* ctx, int e, const char* when) {
  if (!e) return LBDEM_OK;
  std::string m = std::string("device error bits") + when + " " + std::to_string(e) + ":";
  if (e & ERR_TYPE) m += " streaming-type";
  if (e & ERR_NBR_OVERFLOW) m += " neighbour-list-overflow";
  if (e & ERR_CELL_OVERFLOW) m += " cell-overflow";
  if (e & ERR_UNCOVER_CAP) m += " uncover-capacity";
  if (e & ERR_PARTICLE_INDEX) m += " particle-index";
  if (e & ERR_NONFINITE) m += " non-finite";
  if (e & ERR_GRID) m += " particle-outside-grid";
  if (e & ERR_PIPELINE) m += " lattice-copy-pipeline-timeout";
  const int code = (e & ERR_NONFINITE) ? LBDEM_ERR_NONFINITE
                 : (e & (ERR_NBR_OVERFLOW | ERR_CELL_OVERFLOW | ERR_UNCOVER_CAP))
                     ? LBDEM_ERR_OVERFLOW
                     : LBDEM_ERR_DEVICE_STATE;
  return setErr(ctx, code, m);
}

LbArgs lbArgs(lbdem_ctx* c) {
  Device& d = c->d;
  const int P = std::max(c->nPart, 1);
  LbArgs a;
  a.fin = d.f[c->cur];
  a.fout = d.f[1 - c->cur];
  a.nF = d.nF;
  a.mask = d.mask;
  a.solid = d.solid;
  a.objIdx = d.objIdx;
  a.mass = d.mass;
  a.rhoS = d.rhoS;
  a.uS = d.uS;
  a.hS = d.hS;
  a.px0 = d.px0;
  a.px1 = d.px1;
  a.pw1 = d.pw1;
  a.pkd = d.pkd;
  a.pkf = d.pkf;
  a.pFHydro = d.pFHydro;
  a.pMHydro = d.pMHydro;
  a.pSHydro = d.pSHydro;
  a.pFluidVol = d.pFluidVol;
  a.pAccF = d.pAccF;
  a.obj = d.obj;
  a.wallF = d.wallF;
  a.scal = d.scal;
  a.iscal = d.iscal;
  a.uscal = d.uscal;
  a.ifList = d.ifList;
  (void)P;
  return a;
}

// CUDA events around one launch of the main lattice kernel (profiling on).
std::pair<cudaEvent_t, cudaEvent_t>* nextLbEvents(lbdem_ctx* c) {
  if (!c->profiling) return nullptr;
  if (c->lbEventsUsed == c->lbEvents.size()) {
    std::pair<cudaEvent_t, cudaEvent_t> e;
    if (cudaEventCreate(&e.first) != cudaSuccess) return nullptr;
    if (cudaEventCreate(&e.second) != cudaSuccess) return nullptr;
    c->lbEvents.push_back(e);
  }
  return &c->lbEvents[c->lbEventsUsed++];
}

FsArgs fsArgs(lbdem_ctx* c) {
  Device& d = c->d;
  FsArgs a;
  a.fcur = d.f[c->cur];
  a.fold = d.f[1 - c->cur];
  a.nF = d.nF;
  a.mask = d.mask;
  a.solid = d.solid;
  a.objIdx = d.objIdx;
  a.fsflag = d.fsflag;
  a.mass = d.mass;
  a.massNew = d.massNew;
  a.rhoS = d.rhoS;
  a.uS = d.uS;
  a.hS = d.hS;
  a.px0 = d.px0;
  a.px1 = d.px1;
  a.pw1 = d.pw1;
  a.pkd = d.pkd;
  a.pkf = d.pkf;
  a.obj = d.obj;
  a.scal = d.scal;
  a.iscal = d.iscal;
  a.ifList = d.ifList;
  return a;
}

DemArgs demArgs(lbdem_ctx* c) {
  Device& d = c->d;
  DemArgs a;
  a.x0 = d.px0;
  a.x1 = d.px1;
  a.w1 = d.pw1;
  a.xinitY = d.xinitY;
  a.dispY = d.dispY;
  a.r = d.pr;
  a.invm = d.pinvm;
  a.invI = d.pinvI;
  a.FHydro = d.pFHydro;
  a.MHydro = d.pMHydro;
  a.FContact = d.pFContact;
  a.MContact = d.pMContact;
  a.FLub = d.pFLub;
  a.MLub = d.pMLub;
  a.FRep = d.pFRep;
  a.FTotal = d.pFTotal;
  a.MTotal = d.pMTotal;
  a.FGrav = d.pFGrav;
  a.xiw = d.pxiw;
  a.xio = d.pxio;
  a.list[0] = d.plist[0];
  a.list[1] = d.plist[1];
  a.xi[0] = d.pxi[0];
  a.xi[1] = d.pxi[1];
  a.partner = d.partner;
  a.gorder = d.gorder;
  a.pairList = d.pairList;
  a.pairbuf = d.pairbuf;
  a.pairflag = d.pairflag;
  a.slotSum = d.slotSum;
  a.kinf = d.kinf;
  a.pcell = d.pcell;
  a.posf = d.posf;
  a.ppos = d.ppos;
  a.cellCount = d.cellCount;
  a.cellStart = d.cellStart;
  a.cellFill = d.cellFill;
  a.cellParts = d.cellParts;
  a.obj = d.obj;
  a.wallF = d.wallF;
  a.walls = d.walls;
  a.scal = d.scal;
  a.iscal = d.iscal;
  a.uscal = d.uscal;
  a.body = d.body;
  return a;
}

int partGrid(lbdem_ctx* c, int block) {
  return std::max(1, std::min((c->nPart + block - 1) / block, c->smCount * 16));
}

// nbrBuildCells (16 particles per 128-thread block) and nbrPartners (4)
int nbrCellsGrid(lbdem_ctx* c) {
  return std::max(1, std::min((c->nPart + 15) / 16, c->smCount * 16));
}

// Neighbour-list rebuild kernels (gated on the device-side rebuild flag).
int enqueueNeighbourList(lbdem_ctx* ctx) {
  const Consts& k = ctx->k;
  DemArgs a = demArgs(ctx);
  cudaStream_t s = ctx->stream;
  const int pg = partGrid(ctx, 128);
  // only the branch the run uses (fixed at creation; each kernel also checks
  // the device flags and returns unless the list is rebuilt in this step)
  if (!ctx->directList) {
    nbrCellAssign<<<pg, 128, 0, s>>>(k, a);
    nbrCellScan<<<1, 1024, 0, s>>>(k, a);
    nbrCellScatter<<<pg, 128, 0, s>>>(k, a);
    nbrCellSort<<<ctx->gridCells, 128, 0, s>>>(k, a);
    nbrBuildCells<<<nbrCellsGrid(ctx), 128, 0, s>>>(k, a);
  } else {
    nbrBuildDirect<<<pg, 128, 0, s>>>(k, a);
    nbrDirectHistory<<<pg, 128, 0, s>>>(k, a);
  }
  nbrPartners<<<nbrCellsGrid(ctx), 128, 0, s>>>(k, a);  // a warp per particle
  nbrPairList<<<std::max(1, std::min(ctx->nPart * MAX_N / 256 + 1, ctx->smCount * 8)), 256, 0,
                s>>>(k, a);
  return launchErr(ctx, "neighbour list");
}

}  // namespace

// ============================================================================

extern "C" int lbdem_create(const lbdem_config* cfg, const lbdem_options* opt,
                            lbdem_ctx** out) {
  if (!cfg || !out) return LBDEM_ERR_INVALID;
  lbdem_ctx* ctx = new lbdem_ctx();
  *out = ctx;
  const int precision = opt ? opt->precision : LBDEM_PLAIN_FP64;
  ctx->precision = precision;
  ctx->device = opt ? opt->device : 0;
  ctx->check_every = opt ? opt->check_every : 0;
  if (opt && opt->chunks_per_block > 0) ctx->chunksPerBlock = opt->chunks_per_block;
  if (precision != LBDEM_PLAIN_FP64 && precision != LBDEM_MIXED)
    return setErr(ctx, LBDEM_ERR_INVALID, "unknown precision form");
  // ---- validation (the supported subset of the reference's inputs) ----
  if (cfg->lbTopography) return setErr(ctx, LBDEM_ERR_INVALID, "topography is not supported");
  const bool rheology = cfg->rheologyModel != LBDEM_NEWTONIAN || cfg->turbulenceSolve != 0;
  if (cfg->rheologyModel < LBDEM_NEWTONIAN || cfg->rheologyModel > LBDEM_VOELLMY)
    return setErr(ctx, LBDEM_ERR_INVALID, "unknown rheology model");
  if (rheology && precision == LBDEM_MIXED)
    return setErr(ctx, LBDEM_ERR_INVALID,
                  "the mixed form runs NEWTONIAN rheology without turbulence; runs with a "
                  "per-node viscosity use the plain FP64 form");
  if (cfg->n_bodies < 0 || cfg->n_bodies > MAX_BODY || (cfg->n_bodies > 0 && !cfg->bodies))
    return setErr(ctx, LBDEM_ERR_INVALID, "at most 8 bodies, with their body.dat records");
  for (int i = 0; i < 6; ++i)
    if (cfg->boundary[i] < 5 || cfg->boundary[i] > 8)
      return setErr(ctx, LBDEM_ERR_INVALID, "only walls on every face (boundary types 5-8)");
  if (cfg->slipCoefficient < 0.0 || cfg->slipCoefficient > 1.0)
    return setErr(ctx, LBDEM_ERR_INVALID, "slipCoefficient outside [0, 1]");
  if (cfg->unitTime <= 0.0 || cfg->unitLength <= 0.0)
    return setErr(ctx, LBDEM_ERR_INVALID, "unitLength and unitTime must be positive");
  if (cfg->n_objects > MAX_OBJ) return setErr(ctx, LBDEM_ERR_INVALID, "too many objects");
  for (int o = 0; o < cfg->n_objects; ++o)
    if (cfg->objects[o].index != o)
      return setErr(ctx, LBDEM_ERR_INVALID, "object index column must equal its position");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return setErr(ctx, LBDEM_ERR_NO_DEVICE, "no CUDA device");
  if (ctx->device < 0 || ctx->device >= ndev)
    return setErr(ctx, LBDEM_ERR_INVALID, "device ordinal " + std::to_string(ctx->device) +
                                              " out of range (" + std::to_string(ndev) + " devices)");
  // the caller's current device is put back on return
  DeviceScope devScope(ctx->device);
  CK(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
  ctx->stream = ctx->own_stream;
  CK(cudaStreamCreateWithFlags(&ctx->fsStream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->fsFork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->fsDone, cudaEventDisableTiming));
  CK(cudaStreamCreateWithFlags(&ctx->sideStream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->demStream, cudaStreamNonBlocking));
  for (cudaEvent_t* e : {&ctx->prepFork, &ctx->prepDone, &ctx->wallFork, &ctx->wallDone,
                         &ctx->demFork, &ctx->demDone})
    CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  CK(cudaDeviceGetAttribute(&ctx->smCount, cudaDevAttrMultiProcessorCount, ctx->device));
  {
    int perSm = 0;
    CK(cudaFuncSetAttribute(lbStepMixed, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            MIXED_SMEM));
    CK(cudaFuncSetAttribute(uncoverResolve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            UNCOVER_SMEM));
    // the many-run entry points of the same kernels
    CK(cudaFuncSetAttribute(lbStepMixedBatch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            MIXED_SMEM));
    CK(cudaFuncSetAttribute(uncoverResolveBatch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            UNCOVER_SMEM));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, lbStepMixed, MIXED_THREADS,
                                                     MIXED_SMEM));
    ctx->lbMixedBlocks = std::max(1, std::min(perSm, LBDEM_MIXED_MAX_PER_SM)) *
                         std::max(1, ctx->smCount);
  }

  Consts& k = ctx->k;
  std::memset(&k, 0, sizeof(k));
  k.debugFlags = opt ? opt->debug_flags : 0;
  ctx->demSolve = cfg->demSolve != 0;
  ctx->lbSolve = cfg->lbSolve != 0;
  ctx->freeSurface = cfg->freeSurfaceSolve != 0;
  ctx->demInitialRepeat = cfg->demInitialRepeat;
  ctx->fluidHeight = cfg->fluidHeight;
  k.freeSurface = ctx->freeSurface ? 1 : 0;
  k.forceField = cfg->forceFieldSolve != 0;
  // measureUnits::setComposite
  const double L = cfg->unitLength, T = cfg->unitTime, D = cfg->unitDensity;
  k.uLength = L;
  k.uTime = T;
  k.uVolume = L * L * L;
  k.uSpeed = L / T;
  k.uAccel = L / T / T;
  k.uAngVel = 1.0 / T;
  const double uDynVisc = D * L * L / T;
  k.uForce = D * L * L * L * L / T / T;
  k.uTorque = D * L * L * L * L * L / T / T;
  // lattice
  k.X = int(std::floor(cfg->lbSizeX / L + 0.5));
  k.Y = int(std::floor(cfg->lbSizeY / L + 0.5));
  k.Z = int(std::floor(cfg->lbSizeZ / L + 0.5));
  if (k.X < 3 || k.Y < 3 || k.Z < 3) return setErr(ctx, LBDEM_ERR_INVALID, "lattice too small");
  k.N = (long long)k.X * k.Y * k.Z;
  // population planes start on 1 KB boundaries (bulk copies of 256-node chunks)
  k.NP = (k.N + 255) / 256 * 256;
  if (k.NP >= (1ll << 32) / Q) return setErr(ctx, LBDEM_ERR_INVALID, "lattice too large");
  k.sy = k.X;
  k.sz = (long long)k.X * k.Y;
  for (int j = 0; j < Q; ++j) {
    k.nbOff[j] = (int)(CX(j) + CY(j) * k.sy + CZ(j) * k.sz);
    k.pushOff[j] = (unsigned)(j * k.NP + k.nbOff[j]);
  }
  k.initDensity = 1.0;
  k.initVisc = cfg->initVisc / uDynVisc;
  k.omega = 1.0 / (0.5 + 3.0 * k.initVisc);
  k.omegaf = 1.0 - 1.0 / (1.0 + 6.0 * k.initVisc);
  // rheology parameters in lattice units (src/LB.cpp:320-324; turbConst is
  // not scaled; unit.Stress = Density Length^2 / Time^2, src/node.cpp:522)
  k.rheo = cfg->rheologyModel;
  k.turbulence = cfg->turbulenceSolve != 0 ? 1 : 0;
  k.plasticVisc = cfg->plasticVisc / uDynVisc;
  k.yieldStress = cfg->yieldStress / (D * L * L / T / T);
  k.frictionCoef = cfg->frictionCoefFluid;
  k.voellmyCoef = cfg->voellmyConstant / k.uAccel;
  k.turbConst = cfg->turbConst;
  k.mixed = precision == LBDEM_MIXED ? 1 : 0;
  if (k.mixed && k.NP >= (1LL << 31))
    return setErr(ctx, LBDEM_ERR_INVALID, "mixed form: lattice larger than 2^31 nodes");
  k.omegaF = (float)k.omega;
  k.omegafF = (float)k.omegaf;
  k.sLF = (float)(k.uLength * k.uForce);
  k.uForceF = (float)k.uForce;
  k.uTorqueF = (float)k.uTorque;
  k.uVolumeF = (float)k.uVolume;
  k.invLengthF = (float)(1.0 / k.uLength);
  k.invSpeedF = (float)(1.0 / k.uSpeed);
  k.invAngVelF = (float)(1.0 / k.uAngVel);
  // three roundings of 2^-24 relative each on a coordinate below the
  // largest lattice side (a margin of 2 on top)
  k.posErrF = (float)(2.0 * 3.0 * 0x1p-24 * (double)std::max(k.X, std::max(k.Y, k.Z)) + 1e-6);
  for (int a = 0; a < 3; ++a) {
    k.lbF[a] = cfg->lbF[a] / k.uAccel;
    ctx->lbFConfig[a] = k.lbF[a];
    k.lbFf[a] = (float)k.lbF[a];
    k.initVel[a] = cfg->initVelocity[a] / k.uSpeed;
  }
  const unsigned s[3] = {(unsigned)k.X, (unsigned)k.Y, (unsigned)k.Z};
  double phys[3];
  for (int a = 0; a < 3; ++a) phys[a] = double(s[a]) * L;
  double bloc[6][3] = {{0.5 * L, 0, 0}, {double(s[0] - 1.5) * L, 0, 0},
                       {0, 0.5 * L, 0}, {0, double(s[1] - 1.5) * L, 0},
                       {0, 0, 0.5 * L}, {0, 0, double(s[2] - 1.5) * L}};
  const double dirs[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  // DEM::discreteElementInit
  k.demSize[0] = phys[0];
  k.demSize[1] = ctx->freeSurface ? cfg->fluidHeight : phys[1];
  k.demSize[2] = phys[2];
  const double demF[3] = {k.lbF[0] * k.uAccel, k.lbF[1] * k.uAccel, k.lbF[2] * k.uAccel};
  const int P = cfg->n_particles, O = cfg->n_objects;
  ctx->nPart = P;
  ctx->nObj = O;
  k.nPart = P;
  k.nObj = O;
  std::vector<double> hx0(3 * P), hx1(3 * P, 0.0), hw1(3 * P, 0.0), hr(P), hinvm(P), hinvI(P),
      hFG(3 * P);
  double meanR = 0.0, rmax = 0.0;
  for (int i = 0; i < P; ++i) {
    const lbdem_particle_in& q = cfg->particles[i];
    const double r = q.r;
    const double singleMass = 4.0 / 3.0 * cfg->density * PI_D * r * r * r;
    const double m = (unsigned)q.size * singleMass;
    const double I = (unsigned)q.size * 2.0 / 5.0 * singleMass * r * r;
    hr[i] = r;
    hinvm[i] = 1.0 / m;
    hinvI[i] = 1.0 / I;
    for (int a = 0; a < 3; ++a) {
      hx0[a * P + i] = q.x[a];
      hFG[a * P + i] = demF[a] * m;
    }
    meanR += r;
    rmax = rmax > r ? rmax : r;
  }
  if (P > 0) meanR /= double(P);
  k.dt = T / double(1);
  k.k = cfg->linearStiff;
  const double avgMass = 4.0 / 3.0 * cfg->density * PI_D * meanR * meanR * meanR;
  k.c = std::sqrt(avgMass * cfg->linearStiff);
  k.mu = cfg->frictionCoefPart;
  k.kinVisc = cfg->kinVisc;
  k.lubN = cfg->lubNormal;
  k.lubT = cfg->lubTangential;
  k.lubR = cfg->lubRotation;
  k.lubCut = cfg->lubCutoff;
  k.electro = cfg->electroForce;
  k.debye = cfg->debyeLength;
  k.objWaitTime = cfg->objWaitTime;
  std::vector<double> hobj((size_t)std::max(O, 1) * OB_STRIDE, 0.0);
  for (int o = 0; o < O; ++o) {
    const lbdem_object_in& in = cfg->objects[o];
    double* ob = &hobj[(size_t)o * OB_STRIDE];
    const double r = in.r;
    const double m = 4.0 / 3.0 * cfg->objectDensity * PI_D * r * r * r;
    const double I = 2.0 / 5.0 * m * r * r;
    for (int a = 0; a < 3; ++a) {
      ob[OB_X0 + a] = in.x[a];
      ob[OB_X0PREV + a] = in.x[a];
      ob[OB_X1 + a] = in.v[a];
      ob[OB_FGRAV + a] = demF[a] * m;
    }
    ob[OB_R] = r;
    ob[OB_MASS] = m;
    ob[OB_INVM] = 1.0 / m;
    ob[OB_INVI] = 1.0 / I;
    ob[OB_INDEX] = (double)in.index;
    ctx->objIndexField[o] = in.index;
  }
  // bodies, src/DEM.cpp:257-266
  const int B = cfg->n_bodies;
  ctx->nBody = B;
  k.nBody = B;
  k.nonLinType = cfg->nonLinType;
  k.springDamp = cfg->springDamp;
  k.k13 = cfg->k13;
  k.epsilon = cfg->epsilon;
  std::vector<double> hbody((size_t)std::max(B, 1) * BD_STRIDE, 0.0);
  for (int b = 0; b < B; ++b) {
    const lbdem_body_in& in = cfg->bodies[b];
    double* bd = &hbody[(size_t)b * BD_STRIDE];
    const double r = in.r;
    const double m = cfg->bodyDensity * (4.0 / 3.0) * PI_D * (r * r * r);
    for (int a = 0; a < 3; ++a) {
      bd[BD_X0 + a] = in.x[a];
      bd[BD_X1 + a] = in.v[a];
      bd[BD_FGRAV + a] = demF[a] * m;
    }
    bd[BD_R] = r;
    bd[BD_M] = m;
    bd[BD_INVM] = 1.0 / m;
    bd[BD_K] = in.k;
    bd[BD_L0] = in.L0;
    bd[BD_L] = in.L0;
  }
  // walls (DEM::initializeWalls: slip/moving flags of boundary[0] for all)
  std::vector<DeviceWall> hw;
  std::vector<int> hwt;
  for (int i = 0; i < 6; ++i)
    if (cfg->boundary[i] >= 5 && cfg->boundary[i] <= 8) {
      DeviceWall w;
      for (int a = 0; a < 3; ++a) {
        w.p[a] = bloc[i][a];
        w.n[a] = dirs[i][a];
      }
      hw.push_back(w);
      const int b0 = cfg->boundary[0];
      const bool slip = b0 == 5 || b0 == 6, moving = b0 == 6 || b0 == 8;
      hwt.push_back(slip ? (moving ? 6 : 5) : (moving ? 8 : 7));
    }
  ctx->nWall = (int)hw.size();
  k.nWall = ctx->nWall;
  // every wall takes boundary0's slip and moving flags (src/DEM.cpp:430-447)
  k.wallType = hwt.empty() ? 7 : hwt[0];
  k.slipS1 = cfg->slipCoefficient;
  k.slipS2 = 1.0 - cfg->slipCoefficient;
  k.slipS1f = (float)k.slipS1;
  k.slipS2f = (float)k.slipS2;
  // neighbour-list geometry (fixed: radii and the DEM box do not change)
  const double cut = 2.0 * rmax + 2.0;
  const int nl[3] = {(int)(k.demSize[0] / cut), (int)(k.demSize[1] / cut),
                     (int)(k.demSize[2] / cut)};
  const int direct = std::min(nl[0], nl[1]) < 3 ? 1 : 0;
  ctx->directList = direct != 0;
  if (!direct && (long long)nl[0] * nl[1] * nl[2] > MAX_L)
    return setErr(ctx, LBDEM_ERR_OVERFLOW, "more than 100000 neighbour cells");
  {
    auto cap = [&](long long blocks, int most) {
      return (int)std::max(1LL, std::min<long long>(blocks, most));
    };
    const int sm = std::max(1, ctx->smCount);
    // free surface: the interface box is about the free-surface area deep
    ctx->gridFs = cap((long long)k.X * k.Z / 32 + 1, sm * 4);
    // mixed lattice step: one resident wave, but at least chunksPerBlock
    // chunks per block
    ctx->gridLattice = cap(k.NP / MIXED_CHUNK / ctx->chunksPerBlock, ctx->lbMixedBlocks);
    // wall-force sweep: blocks per box face (the largest face's inner nodes)
    const long long face = std::max({(long long)k.Y * k.Z, (long long)k.X * k.Z,
                                     (long long)k.X * k.Y});
    ctx->gridShell = cap(face / 256 + 1, sm * 2);
    long long box = 0;
    for (int o = 0; o < cfg->n_objects; ++o) {
      const long long side = (long long)(2.0 * cfg->objects[o].r / L) + 6;
      box += side * side * side;
    }
    ctx->gridObj = cap(box / 256 + 1, sm * 8);
    const long long cells = direct ? 1 : (long long)nl[0] * nl[1] * nl[2];
    ctx->gridCells = cap(cells / 128 + 1, sm * 8);
  }

  // ---- allocation ----
  Device& d = ctx->d;
  const size_t N = (size_t)k.N;
  const size_t NP = (size_t)k.NP;
  int rc;
#define AL(ptr, n)                                      \
  if ((rc = dalloc(ctx, &(ptr), (n))) != LBDEM_OK) return rc;
  AL(d.mask, NP);  // padded: the lattice step copies whole 256-node chunks
  AL(d.solid, NP);  // padded: the mixed lattice step copies whole chunks
  AL(d.objIdx, N);
  AL(d.claim, N);
  AL(d.fsflag, N);
  if (k.mixed) {
    float* f0 = nullptr;
    float* f1 = nullptr;
    AL(f0, (size_t)Q * NP);
    AL(f1, (size_t)Q * NP);
    d.f[0] = f0;
    d.f[1] = f1;
    AL(d.nF, NP);  // padded: the lattice step copies whole chunks
  } else {
    double* f0 = nullptr;
    double* f1 = nullptr;
    AL(f0, (size_t)Q * NP);
    AL(f1, (size_t)Q * NP);
    d.f[0] = f0;
    d.f[1] = f1;
  }
  AL(d.mass, N);
  AL(d.massNew, N);
  if (rheology) {
    AL(d.visc, N);
    k.visc = d.visc;
  }
  AL(d.rhoS, N);
  AL(d.uS, 3 * N);
  AL(d.hS, 3 * N);
  AL(d.scal, SC_COUNT);
  AL(d.iscal, IS_COUNT);
  AL(d.uscal, US_COUNT);
  const size_t P1 = (size_t)std::max(P, 1);
  AL(d.px0, 3 * P1);
  AL(d.px1, 3 * P1);
  AL(d.pw1, 3 * P1);
  AL(d.pr, P1);
  AL(d.pinvm, P1);
  AL(d.pinvI, P1);
  AL(d.pkd, 6 * P1);
  if (k.mixed) AL(d.pkf, 12 * P1);
  if (k.mixed) AL(d.pAccF, ACCF_STRIDE * P1);
  if (k.mixed) {
    AL(d.chunkAct, NP / 256);
    // every chunk may hold active nodes until the first lattice step checks
    CK(cudaMemsetAsync(d.chunkAct, 0xFF, NP / 256 * sizeof(uint32_t), ctx->stream));
    k.chunkAct = d.chunkAct;
  }
  // hydro accumulators contiguous (reset together each LB step)
  double* hyd = nullptr;
  AL(hyd, 16 * P1);
  d.pFHydro = hyd;
  d.pMHydro = hyd + 3 * P1;
  d.pSHydro = hyd + 6 * P1;
  d.pFluidVol = hyd + 15 * P1;
  AL(d.pFContact, 3 * P1);
  AL(d.pMContact, 3 * P1);
  AL(d.pFLub, 3 * P1);
  AL(d.pMLub, 3 * P1);
  AL(d.pFRep, 3 * P1);
  AL(d.pFTotal, 3 * P1);
  AL(d.pMTotal, 3 * P1);
  AL(d.pFGrav, 3 * P1);
  AL(d.pxiw, 3 * P1);
  AL(d.pxio, 3 * P1);
  AL(d.plist[0], P1 * MAX_N);
  AL(d.plist[1], P1 * MAX_N);
  AL(d.pxi[0], P1 * 3 * MAX_N);
  AL(d.pxi[1], P1 * 3 * MAX_N);
  AL(d.partner, P1 * MAX_N);
  AL(d.gorder, P1 * MAX_N);
  // each owner pair is one slot of one list: at most (MAX_N - 1) / 2 per particle
  AL(d.pairList, (size_t)P1 * (MAX_N / 2));
  // per slot PAIR_VALS doubles (plain form) or floats (mixed form)
  AL(d.pairbuf, P1 * MAX_N * (k.mixed ? PAIR_VALS / 2 : PAIR_VALS));
  AL(d.pairflag, P1 * MAX_N);
  if (k.mixed) {
    AL(d.slotSum, P1 * SLOT_SUM_STRIDE);
    AL(d.kinf, 2 * P1);
  }
  AL(d.pcell, P1);
  AL(d.posf, P1);
  AL(d.ppos, P1);
  AL(d.cellCount, (size_t)MAX_L);
  AL(d.cellStart, (size_t)MAX_L);
  AL(d.cellFill, (size_t)MAX_L);
  AL(d.cellParts, P1);
  AL(d.obj, (size_t)std::max(O, 1) * OB_STRIDE);
  AL(d.body, (size_t)std::max(B, 1) * BD_STRIDE);
  AL(d.wallF, (size_t)MAX_WALL * 12);
  AL(d.walls, (size_t)MAX_WALL);
  AL(d.uncover, (size_t)UNCOVER_CAP);
  AL(d.ifList, N);
  AL(d.stress, (size_t)STRESS_N);
  AL(d.pStress, 9 * P1);
  AL(d.xinitY, P1);
  AL(d.dispY, P1);
  int* dBoundary = nullptr;
  int* dWallType = nullptr;
  AL(dBoundary, 6);
  AL(dWallType, MAX_WALL);
#undef AL
  cudaStream_t st = ctx->stream;
  // ---- uploads ----
  CK(cudaMemcpyAsync(d.px0, hx0.data(), 3 * P * sizeof(double), cudaMemcpyHostToDevice, st));
  // particle::x_i = x0 at the start (src/DEM.cpp:288)
  CK(cudaMemcpyAsync(d.xinitY, d.px0 + P, P * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(d.pr, hr.data(), P * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d.pinvm, hinvm.data(), P * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d.pinvI, hinvI.data(), P * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d.pFGrav, hFG.data(), 3 * P * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d.obj, hobj.data(), hobj.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d.body, hbody.data(), hbody.size() * sizeof(double), cudaMemcpyHostToDevice,
                     st));
  if (!hw.empty()) {
    CK(cudaMemcpyAsync(d.walls, hw.data(), hw.size() * sizeof(DeviceWall), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dWallType, hwt.data(), hwt.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  }
  CK(cudaMemcpyAsync(dBoundary, cfg->boundary, 6 * sizeof(int), cudaMemcpyHostToDevice, st));
  std::vector<int> iscal0(IS_COUNT, 0);
  iscal0[IS_NL] = nl[0];
  iscal0[IS_NL + 1] = nl[1];
  iscal0[IS_NL + 2] = nl[2];
  iscal0[IS_DIRECT] = direct;
  CK(cudaMemcpyAsync(d.iscal, iscal0.data(), IS_COUNT * sizeof(int), cudaMemcpyHostToDevice, st));
  const unsigned long long none = ~0ull;
  CK(cudaMemcpyAsync(d.uscal + US_FIRSTFLAG, &none, sizeof(none), cudaMemcpyHostToDevice, st));
  // ---- LB::latticeBolzmannInit on the device ----
  const int lg = latticeGrid(ctx);
  // every node starts with initVisc (node::initialize)
  if (d.visc) fillDouble<<<lg, 256, 0, st>>>(d.visc, (long long)N, k.initVisc);
  if (ctx->lbSolve) {
    // under lbRestart, LB::initializeTypes without the free-surface
    // interface, then the recycle file (src/LB.cpp:353-367)
    const int fsInit = cfg->lbRestart ? 0 : k.freeSurface;
    initTypes<<<lg, 256, 0, st>>>(k, d.mask, d.solid, d.objIdx, dBoundary, d.walls, dWallType,
                                  d.obj, cfg->fluidHeight / L, fsInit);
    if (!cfg->lbRestart)
      initFields<<<lg, 256, 0, st>>>(k, d.mask, d.f[0], d.mass, d.nF, cfg->fluidHeight / L,
                                     k.freeSurface);
    if ((rc = launchErr(ctx, "lattice init")) != LBDEM_OK) return rc;
    if (cfg->lbRestart && (rc = lbdemRestartFluid(ctx, cfg->lbRestartFile)) != LBDEM_OK)
      return rc;
  }
  // ---- initial neighbour list (DEM::discreteElementInit, :294-296) ----
  {
    DemArgs a = demArgs(ctx);
    demBegin<<<partGrid(ctx, 256), 256, 0, st>>>(k, a, 1);
    if ((rc = enqueueNeighbourList(ctx)) != LBDEM_OK) return rc;
  }
  dfree(ctx, dBoundary);
  dfree(ctx, dWallType);
  if (opt && opt->async_init) return launchErr(ctx, "init");
  CK(cudaStreamSynchronize(st));
  int e = 0;
  CK(cudaMemcpy(&e, d.iscal + IS_ERROR, sizeof(int), cudaMemcpyDeviceToHost));
  return deviceError(ctx, e, " during init");
}

extern "C" void lbdem_destroy(lbdem_ctx* ctx) {
  if (!ctx) return;
  DeviceScope devScope(ctx->device);
  if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& g : ctx->pairGraph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& g : ctx->oneGraph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& row : ctx->groupGraph)
    for (auto& g : row)
      if (g) cudaGraphExecDestroy(g);
  for (auto& e : ctx->lbEvents) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  for (auto& e : ctx->phaseEvents)
    for (cudaEvent_t x : e) cudaEventDestroy(x);
  lbdemOutputDrain(ctx, true);
  lbdemOutputFree(ctx);
  for (auto& b : ctx->buffers) cudaFreeAsync(b.first, ctx->own_stream);
  if (ctx->own_stream) {
    cudaStreamSynchronize(ctx->own_stream);
    cudaStreamDestroy(ctx->own_stream);
  }
  if (ctx->fsStream) {
    cudaStreamSynchronize(ctx->fsStream);
    cudaStreamDestroy(ctx->fsStream);
  }
  if (ctx->fsFork) cudaEventDestroy(ctx->fsFork);
  if (ctx->fsDone) cudaEventDestroy(ctx->fsDone);
  for (cudaStream_t* st : {&ctx->sideStream, &ctx->demStream})
    if (*st) {
      cudaStreamSynchronize(*st);
      cudaStreamDestroy(*st);
    }
  for (cudaEvent_t e : {ctx->prepFork, ctx->prepDone, ctx->wallFork, ctx->wallDone, ctx->demFork,
                        ctx->demDone})
    if (e) cudaEventDestroy(e);
  delete ctx;
}

extern "C" const char* lbdem_last_error(const lbdem_ctx* ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

extern "C" int lbdem_set_stream(lbdem_ctx* ctx, void* stream) {
  if (!ctx) return LBDEM_ERR_INVALID;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return LBDEM_OK;
}

// the stress sums of DEM::evaluateForces, on cycles whose stress-file line
// is due: after the pair pass, before the gather moves the particles
static int enqueueStress(lbdem_ctx* ctx, const DemArgs& a) {
  if (!ctx->stressNext) return LBDEM_OK;
  CK(cudaMemsetAsync(ctx->d.stress, 0, STRESS_N * sizeof(double), ctx->stream));
  double* per = ctx->pStressNext ? ctx->d.pStress : nullptr;
  if (per)
    CK(cudaMemsetAsync(per, 0, 9 * (size_t)std::max(ctx->nPart, 1) * sizeof(double),
                       ctx->stream));
  if (ctx->nPart > 0) {
    demStress<<<partGrid(ctx, 128), 128, 0, ctx->stream>>>(ctx->k, a, ctx->d.pSHydro,
                                                           ctx->d.stress, per);
    ++ctx->launches;
  }
  return LBDEM_OK;
}

// DEM::discreteElementStep (multiStep = 1)
// The DEM step up to its gather (DEM::discreteElementStep: the neighbour
// list check and rebuild, the pair forces, the slot sums) on ctx->stream.
static int enqueueDemPre(lbdem_ctx* ctx) {
  const Consts& k = ctx->k;
  DemArgs a = demArgs(ctx);
  cudaStream_t s = ctx->stream;
  demBegin<<<partGrid(ctx, 256), 256, 0, s>>>(k, a, 0);
  int rc = enqueueNeighbourList(ctx);
  if (rc) return rc;
  const int pairGrid = std::max(1, std::min(ctx->nPart * (MAX_N / 2) / 128 + 1, ctx->smCount * 16));
  if (k.mixed) {
    demPairsMixed<<<pairGrid, 128, 0, s>>>(k, a);
    if ((rc = enqueueStress(ctx, a))) return rc;
    demSlotSumsMixed<<<partGrid(ctx, GATHER_MIXED_PARTS), GATHER_MIXED_THREADS, 0, s>>>(k, a);
  } else {
    demPairs<<<pairGrid, 128, 0, s>>>(k, a);
    if ((rc = enqueueStress(ctx, a))) return rc;
  }
  ctx->launches += 1 + (ctx->directList ? 4 : 7) + (k.mixed ? 2 : 1);
  return LBDEM_OK;
}

extern "C" int lbdem_dem_step(lbdem_ctx* ctx) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  ++ctx->demTimeStep;
  ctx->demTime += ctx->k.dt;
  const Consts& k = ctx->k;
  DemArgs a = demArgs(ctx);
  cudaStream_t s = ctx->stream;
  int rc;
  if (ctx->demPrePending) {  // enqueued beside the previous cycle's lattice step
    CK(cudaStreamWaitEvent(s, ctx->demDone, 0));
    ctx->demPrePending = false;
  } else if ((rc = enqueueDemPre(ctx))) {
    return rc;
  }
  // the gathers also update the impactor (last block)
  if (ctx->wallPendingMain) {  // the gather's last block reads the wall sums
    CK(cudaStreamWaitEvent(s, ctx->wallDone, 0));
    ctx->wallPendingMain = false;
  }
  if (k.mixed) demGatherMixed<<<partGrid(ctx, GATHER_THREADS), GATHER_THREADS, 0, s>>>(k, a);
  else demGather<<<partGrid(ctx, GATHER_THREADS), GATHER_THREADS, 0, s>>>(k, a);
  ctx->launches += 1;
  return launchErr(ctx, "dem step");
}

// LB::latticeBoltzmannCouplingStep
// Start of the lattice step: per-step resets and the kinematics snapshot
// (lbPrepare) on stream st.
static void enqueuePrepare(lbdem_ctx* ctx, cudaStream_t st) {
  Device& d = ctx->d;
  const int P1 = std::max(ctx->nPart, 1);
  lbPrepare<<<std::max(1, std::min(16 * P1 / 256 + 1, 1024)), 256, 0, st>>>(
      ctx->k, d.pFHydro, 16LL * P1, d.pAccF, (long long)ACCF_STRIDE * P1, d.obj, d.wallF, d.scal,
      d.iscal, d.px0, d.px1, d.pw1, d.pkd, d.pkf);
}

extern "C" int lbdem_coupling_step(lbdem_ctx* ctx) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  const Consts& k = ctx->k;
  Device& d = ctx->d;
  cudaStream_t s = ctx->stream;
  const int lg = latticeGrid(ctx);
  if (ctx->overlap && k.mixed && ctx->lbSolve && ctx->demTime >= ctx->demInitialRepeat) {
    // the lattice step's preparation (accumulator resets, kinematics
    // snapshot) touches nothing the coupling kernels read or write
    CK(cudaEventRecord(ctx->prepFork, s));
    CK(cudaStreamWaitEvent(ctx->sideStream, ctx->prepFork, 0));
    enqueuePrepare(ctx, ctx->sideStream);
    CK(cudaEventRecord(ctx->prepDone, ctx->sideStream));
    ctx->prepPending = true;
  }
  if (ctx->nObj > 0) {
    uncoverCollect<<<ctx->gridObj, 256, 0, s>>>(k, d.mask, d.solid, d.obj, d.uncover, d.iscal);
    uncoverResolve<<<1, 1024, UNCOVER_SMEM, s>>>(k, d.mask, d.f[ctx->cur], d.mass, d.nF, d.uncover,
                                      d.iscal);
    voxelizeObjects<<<ctx->gridObj, 256, 0, s>>>(k, d.mask, d.solid, d.objIdx, d.mass, d.obj);
    ctx->launches += 3;
  }
  flagClaim<<<partGrid(ctx, 4) , 128, 0, s>>>(k, d.mask, d.claim, d.px0, d.pr, d.iscal, d.uscal);
  flagApply<<<lg, 256, 0, s>>>(k, d.mask, d.solid, d.claim, d.iscal, d.uscal);
  findNewActiveKernel<<<1, 1024, 0, s>>>(k, d.mask, d.solid, d.px0, d.pr, d.iscal, d.uscal);
  ctx->launches += 3;
  return launchErr(ctx, "coupling step");
}

// LB::latticeBolzmannStep
extern "C" int lbdem_lb_step(lbdem_ctx* ctx) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  if (!ctx->k.forceField && !ctx->lbFReset) {  // LB::collision, src/LB.cpp:1303-1305
    ctx->lbFReset = true;
    ctx->k.lbF[0] = ctx->k.lbF[1] = ctx->k.lbF[2] = 0.0;
    ctx->k.lbFf[0] = ctx->k.lbFf[1] = ctx->k.lbFf[2] = 0.0f;
  }
  const Consts& k = ctx->k;
  Device& d = ctx->d;
  cudaStream_t s = ctx->stream;
  if (ctx->prepPending) {
    CK(cudaStreamWaitEvent(s, ctx->prepDone, 0));
    ctx->prepPending = false;
  } else {
    enqueuePrepare(ctx, s);
  }
  LbArgs a = lbArgs(ctx);
  auto* ev = nextLbEvents(ctx);
  if (ev) cudaEventRecord(ev->first, s);
  if (k.mixed)
    lbStepMixed<<<ctx->gridLattice,
                  MIXED_THREADS, MIXED_SMEM, s>>>(k, a);
  else if (k.visc) lbStepFp64Rheo<<<ctx->smCount * 4, 256, 0, s>>>(k, a);
  else lbStepFp64<<<ctx->smCount * 4, 256, 0, s>>>(k, a);
  if (ev) cudaEventRecord(ev->second, s);
  if (k.mixed && k.nWall > 0 && k.wallType >= 7) {
    if (ctx->overlap) {
      CK(cudaEventRecord(ctx->wallFork, s));
      CK(cudaStreamWaitEvent(ctx->sideStream, ctx->wallFork, 0));
      lbWallForceMixed<<<dim3(ctx->gridShell, 6), 256, 0, ctx->sideStream>>>(k, a);
      CK(cudaEventRecord(ctx->wallDone, ctx->sideStream));
      ctx->wallPendingFs = ctx->wallPendingMain = true;
    } else {
      lbWallForceMixed<<<dim3(ctx->gridShell, 6), 256, 0, s>>>(k, a);
    }
    ctx->launches += 1;
  }
  if (k.wallType == 5 || k.wallType == 6) {
    // slip walls: the diagonal links' slip rule, after every node has streamed
    slipStash<<<latticeGrid(ctx), 256, 0, s>>>(k, d.mask, a.fout);
    slipApply<<<latticeGrid(ctx), 256, 0, s>>>(k, d.mask, a.fout);
    ctx->launches += 2;
  }
  ctx->cur = 1 - ctx->cur;
  // unit conversions, then the extra-mass redistribution (free surface)
  lbFinalizeKernel<<<std::max(ctx->gridFs, partGrid(ctx, 256)), 256, 0, s>>>(
      k, d.pFHydro, d.pMHydro, d.pFluidVol, d.obj, d.wallF, d.scal, d.iscal, d.pAccF, d.pSHydro,
      fsArgs(ctx), ctx->freeSurface ? 1 : 0);
  ctx->launches += 3;
  return launchErr(ctx, "lb step");
}

// LB::latticeBoltzmannFreeSurfaceStep
extern "C" int lbdem_free_surface_step(lbdem_ctx* ctx) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  const Consts& k = ctx->k;
  Device& d = ctx->d;
  cudaStream_t s = ctx->stream;
  const int g = ctx->gridFs;
  FsArgs a = fsArgs(ctx);
  fsUpdateMass<<<g, 256, 0, s>>>(k, a);
  if (ctx->wallPendingFs) {  // the wall sweep reads node types that fsMutants changes
    CK(cudaStreamWaitEvent(s, ctx->wallDone, 0));
    ctx->wallPendingFs = false;
  }
  fsMutants<<<g, 256, 0, s>>>(k, a);
  fsSmoothen<<<g, 256, 0, s>>>(k, a);
  fsMutantsAndFill<<<g, 256, 0, s>>>(k, a);
  fsEmptyIsolated<<<g, 256, 0, s>>>(k, a);
  fsRedistribute<<<g, 256, 0, s>>>(k, a);
  ctx->launches += 6;
  return launchErr(ctx, "free-surface step");
}

extern "C" int lbdem_profile_enable(lbdem_ctx* ctx, int enable) {
  if (!ctx) return LBDEM_ERR_INVALID;
  ctx->profiling = enable != 0;
  return LBDEM_OK;
}

extern "C" int lbdem_profile_read(lbdem_ctx* ctx, lbdem_profile* out, int reset) {
  if (!ctx || !out) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  std::memset(out, 0, sizeof(*out));
  CK(cudaStreamSynchronize(ctx->stream));
  double ms = 0.0;
  for (size_t i = 0; i < ctx->lbEventsUsed; ++i) {
    float t = 0.0f;
    CK(cudaEventElapsedTime(&t, ctx->lbEvents[i].first, ctx->lbEvents[i].second));
    ms += t;
  }
  unsigned long long upd = 0;
  CK(cudaMemcpy(&upd, ctx->d.uscal + US_ACTIVE_UPDATES, sizeof(upd), cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < ctx->phaseEventsUsed; ++i)
    for (int p = 0; p < 4; ++p) {
      float t = 0.0f;
      CK(cudaEventElapsedTime(&t, ctx->phaseEvents[i][p], ctx->phaseEvents[i][p + 1]));
      out->phase_ms[p] += t;
    }
  out->lb_kernel_ms = ms;
  out->lb_kernel_launches = (int64_t)ctx->lbEventsUsed;
  out->kernel_launches = ctx->launches;
  out->active_node_updates = (int64_t)upd;
  if (reset) {
    ctx->lbEventsUsed = 0;
    ctx->phaseEventsUsed = 0;
    ctx->launches = 0;
    CK(cudaMemsetAsync(ctx->d.uscal + US_ACTIVE_UPDATES, 0, sizeof(upd), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return LBDEM_OK;
}

// goCycle, src/main.cpp:38-67 (without IO)
namespace {

// One goCycle (src/main.cpp:38-67) without IO.
// Events at the step boundaries of a profiled cycle (profiling on).
cudaEvent_t* nextPhaseEvents(lbdem_ctx* c) {
  if (!c->profiling) return nullptr;
  if (c->phaseEventsUsed == c->phaseEvents.size()) {
    std::array<cudaEvent_t, 5> e;
    for (auto& x : e)
      if (cudaEventCreate(&x) != cudaSuccess) return nullptr;
    c->phaseEvents.push_back(e);
  }
  return c->phaseEvents[c->phaseEventsUsed++].data();
}

// The next cycle's coupling step (and whatever follows the DEM step) waits
// for a forked free-surface step.
int joinFreeSurface(lbdem_ctx* ctx) {
  if (!ctx->fsPending) return LBDEM_OK;
  ctx->fsPending = false;
  CK(cudaStreamWaitEvent(ctx->stream, ctx->fsDone, 0));
  return LBDEM_OK;
}

// One goCycle. With forkFs (mixed form, inside a capture of several cycles)
// the free-surface step goes to fsStream after the lattice step and the
// next cycle's DEM step runs beside it: that DEM step reads the particle
// state and the hydrodynamic sums of the lattice step, and the free-surface
// step of the mixed form reads only the lattice and the kinematics snapshot
// taken at the start of the lattice step.
int cycleOnce(lbdem_ctx* ctx, bool forkFs = false) {
  {
    ++ctx->lbTime;
    int rc = LBDEM_OK;
    cudaEvent_t* pe = nextPhaseEvents(ctx);
    int marked = 0;  // events recorded so far; steps not taken get zero time
    auto mark = [&](int i) {
      for (; pe && marked <= i; ++marked) cudaEventRecord(pe[marked], ctx->stream);
    };
    mark(0);
    if (ctx->demSolve && (rc = lbdem_dem_step(ctx))) return rc;
    if ((rc = joinFreeSurface(ctx))) return rc;
    mark(1);
    if (ctx->lbSolve && ctx->demTime >= ctx->demInitialRepeat) {
      if (ctx->demSolve && (rc = lbdem_coupling_step(ctx))) return rc;
      if (forkFs && ctx->overlap && ctx->demSolve && !ctx->out) {
        // the next cycle's DEM step up to its gather reads only particle
        // state, which nothing from here to that gather changes, and writes
        // only DEM data: it runs beside this cycle's lattice step
        CK(cudaEventRecord(ctx->demFork, ctx->stream));
        CK(cudaStreamWaitEvent(ctx->demStream, ctx->demFork, 0));
        cudaStream_t main = ctx->stream;
        ctx->stream = ctx->demStream;
        rc = enqueueDemPre(ctx);
        ctx->stream = main;
        if (rc) return rc;
        CK(cudaEventRecord(ctx->demDone, ctx->demStream));
        ctx->demPrePending = true;
      }
      mark(2);
      if ((rc = lbdem_lb_step(ctx))) return rc;
      mark(3);
      if (ctx->freeSurface && forkFs && ctx->k.mixed) {
        CK(cudaEventRecord(ctx->fsFork, ctx->stream));
        CK(cudaStreamWaitEvent(ctx->fsStream, ctx->fsFork, 0));
        cudaStream_t main = ctx->stream;
        ctx->stream = ctx->fsStream;
        rc = lbdem_free_surface_step(ctx);
        ctx->stream = main;
        if (rc) return rc;
        CK(cudaEventRecord(ctx->fsDone, ctx->fsStream));
        ctx->fsPending = true;
      } else if (ctx->freeSurface && (rc = lbdem_free_surface_step(ctx))) {
        return rc;
      }
      mark(4);
    } else if (ctx->lbSolve && ctx->demTime <= ctx->demInitialRepeat) {
      if (ctx->demSolve && (rc = lbdem_coupling_step(ctx))) return rc;
    }
    mark(4);
    if (ctx->check_every > 0 && ctx->lbTime % ctx->check_every == 0 && ctx->lbSolve) {
      nonfiniteCheck<<<latticeGrid(ctx), 256, 0, ctx->stream>>>(
          ctx->k, ctx->d.mask, ctx->d.f[ctx->cur], ctx->d.iscal);
      ++ctx->launches;
    }
  }
  return LBDEM_OK;
}

// Two goCycles launch the same kernels with the same arguments whenever
// nothing decided on the host changes between them: the lattice buffers
// swap twice, the DEM step number lives on the device, and Consts is fixed
// once the first collision has applied the reference's force reset. Such
// pairs are replayed from a CUDA graph (one per starting buffer), which
// takes the per-kernel launch cost off the host.
bool pairReplayable(const lbdem_ctx* ctx) {
  if (ctx->check_every > 0 || ctx->profiling) return false;
  if (ctx->lbSolve && !ctx->k.forceField && !ctx->lbFReset) return false;
  // the branch on demTime of goCycle is settled for both cycles
  if (ctx->lbSolve && ctx->demSolve && !(ctx->demTime + ctx->k.dt >= ctx->demInitialRepeat))
    return false;
  return true;
}

// Captures `cycles` (1 or 2) consecutive cycles into *exec and launches it
// once: the capture advanced the host counters, the first replay is the
// cycles themselves.
int captureCycles(lbdem_ctx* ctx, int cycles, cudaGraphExec_t* exec, long long* kernels) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  const long long before = ctx->launches;
  int rc = LBDEM_OK;
  ctx->overlap = ctx->k.mixed != 0;
  for (int c = 0; c < cycles && rc == LBDEM_OK; ++c) rc = cycleOnce(ctx, c + 1 < cycles);
  ctx->overlap = false;
  // the capture ends on the context's stream with every fork joined
  const int rj = joinFreeSurface(ctx);
  if (rc == LBDEM_OK) rc = rj;
  if (ctx->demPrePending) {  // not expected: the last cycle forks no DEM step
    const cudaError_t ew = cudaStreamWaitEvent(ctx->stream, ctx->demDone, 0);
    if (rc == LBDEM_OK && ew != cudaSuccess) rc = setErr(ctx, LBDEM_ERR_CUDA, "graph capture join");
    ctx->demPrePending = false;
  }
  if (ctx->wallPendingMain || ctx->wallPendingFs || ctx->prepPending) {
    const cudaEvent_t e = ctx->prepPending ? ctx->prepDone : ctx->wallDone;
    const cudaError_t ew = cudaStreamWaitEvent(ctx->stream, e, 0);
    if (rc == LBDEM_OK && ew != cudaSuccess) rc = setErr(ctx, LBDEM_ERR_CUDA, "graph capture join");
    ctx->wallPendingMain = ctx->wallPendingFs = ctx->prepPending = false;
  }
  const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return setErr(ctx, LBDEM_ERR_CUDA, std::string("graph capture: ") +
                                                               cudaGetErrorString(e));
  const cudaError_t ei = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess)
    return setErr(ctx, LBDEM_ERR_CUDA, std::string("graph instantiate: ") +
                                           cudaGetErrorString(ei));
  *kernels = ctx->launches - before;
  CK(cudaGraphLaunch(*exec, ctx->stream));
  return LBDEM_OK;
}

int capturePair(lbdem_ctx* ctx, int parity) {
  return captureCycles(ctx, 2, &ctx->pairGraph[parity], &ctx->pairKernels);
}

}  // namespace

// ---- many runs advanced by one launch per kernel ----------------------------

// The record of run c for a cycle that starts on lattice buffer cur: the
// lattice step reads buffer cur, the finalisation and the free-surface step
// (after the swap) see 1 - cur as current.
void lbdemJobArgs(lbdem_ctx* c, int cur, JobArgs* j) {
  std::memset(j, 0, sizeof *j);
  const int save = c->cur;
  c->cur = cur;
  j->k = c->k;
  j->dem = demArgs(c);
  j->lb = lbArgs(c);
  c->cur = 1 - cur;
  j->fs = fsArgs(c);
  c->cur = save;
  Device& d = c->d;
  CoupArgs& p = j->cp;
  p.mask = d.mask;
  p.solid = d.solid;
  p.objIdx = d.objIdx;
  p.claim = d.claim;
  p.mass = d.mass;
  p.nF = d.nF;
  p.fcur = d.f[cur];
  p.uncover = d.uncover;
  p.px0 = d.px0;
  p.px1 = d.px1;
  p.pw1 = d.pw1;
  p.pr = d.pr;
  p.obj = d.obj;
  p.wallF = d.wallF;
  p.scal = d.scal;
  p.iscal = d.iscal;
  p.uscal = d.uscal;
  const long long P1 = std::max(c->nPart, 1);
  p.pAcc = d.pFHydro;
  p.pAccLen = 16LL * P1;
  p.pAccF = d.pAccF;
  p.pAccFLen = (long long)ACCF_STRIDE * P1;
  p.pkd = d.pkd;
  p.pkf = d.pkf;
  p.pF = d.pFHydro;
  p.pM = d.pMHydro;
  p.pV = d.pFluidVol;
  p.pS = d.pSHydro;
  p.redistribute = c->freeSurface ? 1 : 0;
}

// Runs whose next two cycles are the steady goCycle (the pair-replay
// conditions) with the DEM, lattice and coupling steps all on; two such runs
// share a batch when their switches match (batchKey).
bool lbdemBatchable(const lbdem_ctx* c) {
  // runs with a per-node viscosity or bodies keep their own launches
  return c->demSolve && c->lbSolve && pairReplayable(c) && !c->k.visc && c->nBody == 0 &&
         c->k.wallType >= 7;
}
int lbdemEnqueueErrorRead(lbdem_ctx* c, int* dst, cudaStream_t st) {
  const int n3 = 3 * c->nPart;
  const int blocks = std::max(1, std::min((n3 + 255) / 256, 64));
  motionFiniteCheck<<<blocks, 256, 0, st>>>(c->d.px0, c->d.px1, c->d.pFHydro, n3, c->d.obj,
                                           c->nObj, c->d.scal, c->d.iscal);
  if (cudaGetLastError() != cudaSuccess) return LBDEM_ERR_CUDA;
  return cudaMemcpyAsync(dst, c->d.iscal + IS_ERROR, sizeof(int), cudaMemcpyDeviceToHost, st) ==
                 cudaSuccess
             ? LBDEM_OK
             : LBDEM_ERR_CUDA;
}
int lbdemErrorStatus(lbdem_ctx* c, int bits, const char* when) {
  return deviceError(c, bits, when);
}
int lbdemBatchKey(const lbdem_ctx* c) {
  return c->precision | (c->freeSurface ? 2 : 0) | (c->nObj > 0 ? 4 : 0) | (c->nWall > 0 ? 8 : 0);
}

// One goCycle of every run (DEM, coupling, lattice, free-surface step, as
// cycleOnce enqueues them) with one launch per kernel: grid z = run, grid
// x = the largest of the runs' own grids (the kernels loop over their work
// by grid stride). jobs: the runs' records for this cycle, on the device.
int lbdemEnqueueBatchCycle(const std::vector<lbdem_ctx*>& runs, const JobArgs* jobs,
                           cudaStream_t s) {
  const unsigned n = (unsigned)runs.size();
  lbdem_ctx* r0 = runs[0];
  auto gmax = [&](auto grid) {
    int g = 1;
    for (lbdem_ctx* c : runs) g = std::max(g, (int)grid(c));
    return g;
  };
  auto G = [&](int gx) { return dim3((unsigned)gx, 1, n); };
  const bool mixed = r0->k.mixed != 0;
  // DEM step
  demBeginBatch<<<G(gmax([](lbdem_ctx* c) { return partGrid(c, 256); })), 256, 0, s>>>(jobs);
  const int pg = gmax([](lbdem_ctx* c) { return partGrid(c, 128); });
  nbrCellAssignBatch<<<G(pg), 128, 0, s>>>(jobs);
  nbrCellScanBatch<<<G(1), 1024, 0, s>>>(jobs);
  nbrCellScatterBatch<<<G(pg), 128, 0, s>>>(jobs);
  nbrCellSortBatch<<<G(gmax([](lbdem_ctx* c) { return c->gridCells; })), 128, 0, s>>>(jobs);
  nbrBuildCellsBatch<<<G(gmax([](lbdem_ctx* c) { return nbrCellsGrid(c); })), 128, 0, s>>>(jobs);
  nbrBuildDirectBatch<<<G(pg), 128, 0, s>>>(jobs);
  nbrDirectHistoryBatch<<<G(pg), 128, 0, s>>>(jobs);
  nbrPartnersBatch<<<G(gmax([](lbdem_ctx* c) { return nbrCellsGrid(c); })), 128, 0, s>>>(jobs);
  nbrPairListBatch<<<G(gmax([](lbdem_ctx* c) {
                       return std::max(1, std::min(c->nPart * MAX_N / 256 + 1, c->smCount * 8));
                     })),
                     256, 0, s>>>(jobs);
  const int pairG = gmax([](lbdem_ctx* c) {
    return std::max(1, std::min(c->nPart * (MAX_N / 2) / 128 + 1, c->smCount * 16));
  });
  const int gathG = gmax([](lbdem_ctx* c) { return partGrid(c, GATHER_THREADS); });
  if (mixed) {
    const int sumG = gmax([](lbdem_ctx* c) { return partGrid(c, GATHER_MIXED_PARTS); });
    demPairsMixedBatch<<<G(pairG), 128, 0, s>>>(jobs);
    demSlotSumsMixedBatch<<<G(sumG), GATHER_MIXED_THREADS, 0, s>>>(jobs);
    demGatherMixedBatch<<<G(gathG), GATHER_THREADS, 0, s>>>(jobs);
  } else {
    demPairsBatch<<<G(pairG), 128, 0, s>>>(jobs);
    demGatherBatch<<<G(gathG), GATHER_THREADS, 0, s>>>(jobs);
  }
  // coupling step
  if (r0->nObj > 0) {
    const int og = gmax([](lbdem_ctx* c) { return c->gridObj; });
    uncoverCollectBatch<<<G(og), 256, 0, s>>>(jobs);
    uncoverResolveBatch<<<G(1), 1024, UNCOVER_SMEM, s>>>(jobs);
    voxelizeObjectsBatch<<<G(og), 256, 0, s>>>(jobs);
  }
  flagClaimBatch<<<G(gmax([](lbdem_ctx* c) { return partGrid(c, 4); })), 128, 0, s>>>(jobs);
  flagApplyBatch<<<G(gmax([](lbdem_ctx* c) { return latticeGrid(c); })), 256, 0, s>>>(jobs);
  findNewActiveKernelBatch<<<G(1), 1024, 0, s>>>(jobs);
  // lattice step
  lbPrepareBatch<<<G(gmax([](lbdem_ctx* c) {
                     return std::max(1, std::min(16 * std::max(c->nPart, 1) / 256 + 1, 1024));
                   })),
                   256, 0, s>>>(jobs);
  if (mixed) {
    lbStepMixedBatch<<<G(gmax([](lbdem_ctx* c) {
                         return c->gridLattice;
                       })),
                       MIXED_THREADS, MIXED_SMEM, s>>>(jobs);
    if (r0->nWall > 0)
      lbWallForceMixedBatch<<<dim3((unsigned)gmax([](lbdem_ctx* c) { return c->gridShell; }), 6,
                                   n),
                              256, 0, s>>>(jobs);
  } else {
    lbStepFp64Batch<<<G(gmax([](lbdem_ctx* c) { return c->smCount * 4; })), 256, 0, s>>>(jobs);
  }
  lbFinalizeKernelBatch<<<G(gmax([](lbdem_ctx* c) {
                            return std::max(c->gridFs, partGrid(c, 256));
                          })),
                          256, 0, s>>>(jobs);
  // free-surface step
  if (r0->freeSurface) {
    const int fg = gmax([](lbdem_ctx* c) { return c->gridFs; });
    fsUpdateMassBatch<<<G(fg), 256, 0, s>>>(jobs);
    fsMutantsBatch<<<G(fg), 256, 0, s>>>(jobs);
    fsSmoothenBatch<<<G(fg), 256, 0, s>>>(jobs);
    fsMutantsAndFillBatch<<<G(fg), 256, 0, s>>>(jobs);
    fsEmptyIsolatedBatch<<<G(fg), 256, 0, s>>>(jobs);
    fsRedistributeBatch<<<G(fg), 256, 0, s>>>(jobs);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return setErr(r0, LBDEM_ERR_CUDA, std::string("batched cycle: ") +
                                                          cudaGetErrorString(e));
  return LBDEM_OK;
}

// Host counters of a run after `cycles` batched cycles (an even number:
// the lattice buffer is back where it started).
void lbdemAdvanceCounters(lbdem_ctx* c, int cycles) {
  for (int i = 0; i < cycles; ++i) {
    ++c->lbTime;
    if (c->demSolve) {
      ++c->demTimeStep;
      c->demTime += c->k.dt;
    }
  }
  if (cycles & 1) c->cur = 1 - c->cur;
}

extern "C" int lbdem_cycle(lbdem_ctx* ctx, int32_t n) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  int32_t i = 0;
  while (i < n) {
    int rc = LBDEM_OK;
    // with no output open, groups of steady cycles are replayed from one
    // graph: LBDEM_GRAPH_CYCLES of them for a call of many cycles, 4 for a
    // short call (a run's first replay of a group captures it: short runs
    // would pay more for capturing long groups than they save); in the mixed
    // form each cycle but the last overlaps its lattice and free-surface
    // steps with the next cycle's DEM step
    const int big = (n >= 4 * LBDEM_GRAPH_CYCLES) ? 1 : 0;
    const int G = big ? LBDEM_GRAPH_CYCLES : 4;
    if (n - i >= G && !ctx->out && pairReplayable(ctx)) {
      const int parity = ctx->cur;
      if (!ctx->groupGraph[big][parity]) {
        if ((rc = captureCycles(ctx, G, &ctx->groupGraph[big][parity], &ctx->groupKernels[big])))
          return rc;
      } else {
        CK(cudaGraphLaunch(ctx->groupGraph[big][parity], ctx->stream));
        // host counters as the cycles advance them (an even number of
        // buffer swaps)
        for (int c = 0; c < G; ++c) {
          ++ctx->lbTime;
          if (ctx->demSolve) {
            ++ctx->demTimeStep;
            ctx->demTime += ctx->k.dt;
          }
        }
        ctx->launches += ctx->groupKernels[big];
      }
      i += G;
      continue;
    }
    // a pair replays two cycles; an output line due after the first of them
    // needs that cycle on its own
    if (n - i >= 2 && pairReplayable(ctx) && !lbdemOutputBlocksPair(ctx)) {
      const int parity = ctx->cur;
      if (!ctx->pairGraph[parity]) {
        if ((rc = capturePair(ctx, parity))) return rc;
      } else {
        CK(cudaGraphLaunch(ctx->pairGraph[parity], ctx->stream));
        // host counters as two cycles advance them (cur flips twice)
        for (int c = 0; c < 2; ++c) {
          ++ctx->lbTime;
          if (ctx->demSolve) {
            ++ctx->demTimeStep;
            ctx->demTime += ctx->k.dt;
          }
        }
        ctx->launches += ctx->pairKernels;
      }
      for (int c = 0; c < 2; ++c)
        if ((rc = lbdemOutputAfterCycle(ctx))) return rc;
      i += 2;
      continue;
    }
    ctx->stressNext = lbdemOutputStressNext(ctx);
    ctx->pStressNext = lbdemOutputParticleStressNext(ctx);
    if (!ctx->stressNext && !ctx->pStressNext && pairReplayable(ctx)) {
      // a single steady cycle: replayed from its own graph (one per starting
      // buffer), as pairs are
      const int parity = ctx->cur;
      if (!ctx->oneGraph[parity]) {
        rc = captureCycles(ctx, 1, &ctx->oneGraph[parity], &ctx->oneKernels);
      } else {
        const cudaError_t e = cudaGraphLaunch(ctx->oneGraph[parity], ctx->stream);
        if (e != cudaSuccess)
          rc = setErr(ctx, LBDEM_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
        // the host counters as cycleOnce advances them (the lattice step,
        // which swaps the buffers, runs once the DEM time reaches
        // demInitialRepeat)
        const double demTimeAfter = ctx->demTime + (ctx->demSolve ? ctx->k.dt : 0.0);
        const bool lbRuns = ctx->lbSolve && demTimeAfter >= ctx->demInitialRepeat;
        ++ctx->lbTime;
        if (ctx->demSolve) {
          ++ctx->demTimeStep;
          ctx->demTime += ctx->k.dt;
        }
        if (lbRuns) ctx->cur = 1 - ctx->cur;
        ctx->launches += ctx->oneKernels;
      }
    } else {
      rc = cycleOnce(ctx);
    }
    ctx->stressNext = ctx->pStressNext = false;
    if (rc) return rc;
    if ((rc = lbdemOutputAfterCycle(ctx))) return rc;
    ++i;
  }
  return lbdemOutputDrain(ctx, false);
}

namespace {
// Pinned host staging for the small record downloads, one block per host
// thread, taken on first use and kept for the life of the process (a
// cudaFreeHost could wait for the whole device, which runs sharing the GPU
// must not do).
constexpr size_t SMALL_READ_BYTES = 64 * 1024;
thread_local unsigned char* t_stage = nullptr;

// lbdem_sync followed by a read of `bytes` bytes at device address src into
// dst, in one host round trip: the error word and the record are copied
// into pinned staging behind the stream's work, then the stream is waited
// for once. Larger records take the two-step path.
int syncAndRead(lbdem_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (bytes + 16 > SMALL_READ_BYTES) {
    if (int rc = lbdem_sync(ctx)) return rc;
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return LBDEM_OK;
  }
  if (!t_stage && cudaHostAlloc((void**)&t_stage, SMALL_READ_BYTES, cudaHostAllocPortable) !=
                      cudaSuccess) {
    t_stage = nullptr;
    if (int rc = lbdem_sync(ctx)) return rc;
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return LBDEM_OK;
  }
  int* err = reinterpret_cast<int*>(t_stage);
  CK(cudaMemcpyAsync(err, ctx->d.iscal + IS_ERROR, sizeof(int), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaMemcpyAsync(t_stage + 16, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (int rc = lbdemOutputDrain(ctx, true)) return rc;
  if (int rc = deviceError(ctx, *err, "")) return rc;
  std::memcpy(dst, t_stage + 16, bytes);
  return LBDEM_OK;
}
}  // namespace

extern "C" int lbdem_sync(lbdem_ctx* ctx) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream));
  if (int rc = lbdemOutputDrain(ctx, true)) return rc;
  int e = 0;
  CK(cudaMemcpy(&e, ctx->d.iscal + IS_ERROR, sizeof(int), cudaMemcpyDeviceToHost));
  return deviceError(ctx, e, "");
}

// Device bytes lbdem_create allocates for cfg, array by array as it does
// (each allocation rounded up to the allocator's 512-byte granularity).
extern "C" int lbdem_estimate_device_bytes(const lbdem_config* cfg, int32_t precision,
                                           int64_t* bytes) {
  if (!cfg || !bytes || cfg->unitLength <= 0.0) return LBDEM_ERR_INVALID;
  if (precision != LBDEM_PLAIN_FP64 && precision != LBDEM_MIXED) return LBDEM_ERR_INVALID;
  const double L = cfg->unitLength;
  const long long X = (long long)std::floor(cfg->lbSizeX / L + 0.5),
                  Y = (long long)std::floor(cfg->lbSizeY / L + 0.5),
                  Z = (long long)std::floor(cfg->lbSizeZ / L + 0.5);
  if (X < 3 || Y < 3 || Z < 3) return LBDEM_ERR_INVALID;
  const long long N = X * Y * Z, NP = (N + 255) / 256 * 256;
  const long long P1 = std::max(cfg->n_particles, 1), O1 = std::max(cfg->n_objects, 1);
  const bool mixed = precision == LBDEM_MIXED;
  long long total = 0;
  auto add = [&](long long n, long long elem) {
    total += (std::max(n, 1LL) * elem + 511) / 512 * 512;
  };
  // lattice
  add(NP, 1);                       // mask
  add(NP, 4);                       // solid
  add(N, 1);                        // objIdx
  add(N, 4);                        // claim
  add(N, 1);                        // fsflag
  add((long long)Q * NP, mixed ? 4 : 8);
  add((long long)Q * NP, mixed ? 4 : 8);
  if (mixed) add(NP, 4);            // nF
  for (int i = 0; i < 2; ++i) add(N, 8);  // mass, massNew
  if (cfg->rheologyModel != LBDEM_NEWTONIAN || cfg->turbulenceSolve) add(N, 8);  // visc
  add(N, 8);                        // rhoS
  add(3 * N, 8);                    // uS
  add(3 * N, 8);                    // hS
  add(SC_COUNT, 8);
  add(IS_COUNT, 4);
  add(US_COUNT, 8);
  // particles
  for (int i = 0; i < 3; ++i) add(3 * P1, 8);  // x0, x1, w1
  for (int i = 0; i < 3; ++i) add(P1, 8);      // r, invm, invI
  add(6 * P1, 8);                              // pkd
  if (mixed) {
    add(12 * P1, 4);                           // pkf
    add(ACCF_STRIDE * P1, 4);                  // pAccF
    add(NP / 256, 4);                          // chunkAct
  }
  add(16 * P1, 8);                             // FHydro, MHydro, SHydro, fluidVolume
  for (int i = 0; i < 10; ++i) add(3 * P1, 8); // contact .. xio
  add(P1 * MAX_N, 4);
  add(P1 * MAX_N, 4);                          // lists
  add(P1 * 3 * MAX_N, 8);
  add(P1 * 3 * MAX_N, 8);                      // tangential springs
  add(P1 * MAX_N, 4);                          // partner
  add(P1 * MAX_N, 4);                          // gorder
  add(P1 * (MAX_N / 2), 4);                    // pairList
  add(P1 * MAX_N * (mixed ? PAIR_VALS / 2 : PAIR_VALS), 8);  // pairbuf
  add(P1 * MAX_N, 1);                          // pairflag
  if (mixed) add(P1 * SLOT_SUM_STRIDE, 4);     // slotSum
  if (mixed) add(2 * P1, 16);                  // kinf
  add(P1, 4);
  add(P1, 4);                                  // pcell, ppos
  add(P1, 16);                                 // posf
  for (int i = 0; i < 3; ++i) add(MAX_L, 4);   // cell arrays
  add(P1, 4);                                  // cellParts
  add(O1 * OB_STRIDE, 8);
  add((long long)std::max(cfg->n_bodies, 1) * BD_STRIDE, 8);
  add(MAX_WALL * 12, 8);
  add(MAX_WALL, (long long)sizeof(DeviceWall));
  add(UNCOVER_CAP, 4);
  add(N, 4);                                   // interface list
  add(STRESS_N, 8);                            // stress sums
  add(9 * P1, 8);                              // per-particle stresslets
  add(2 * P1, 8);                              // x_i.y, disp.y
  *bytes = total;
  return LBDEM_OK;
}

static std::atomic<int64_t> g_deviceAllocations{0};

void lbdemNoteDeviceAllocation() { g_deviceAllocations.fetch_add(1, std::memory_order_relaxed); }

extern "C" int64_t lbdem_device_allocations(void) {
  return g_deviceAllocations.load(std::memory_order_relaxed);
}

extern "C" int lbdem_get_info(lbdem_ctx* ctx, lbdem_info* info) {
  if (!ctx || !info) return LBDEM_ERR_INVALID;
  std::memset(info, 0, sizeof(*info));
  info->lb_size[0] = ctx->k.X;
  info->lb_size[1] = ctx->k.Y;
  info->lb_size[2] = ctx->k.Z;
  info->nodes = ctx->k.N;
  info->n_particles = ctx->nPart;
  info->n_objects = ctx->nObj;
  info->n_walls = ctx->nWall;
  info->precision = ctx->precision;
  info->time_step = ctx->lbTime;
  info->dem_step = ctx->demTimeStep;
  info->dem_time = ctx->demTime;
  info->unit_length = ctx->k.uLength;
  info->unit_time = ctx->k.uTime;
  info->device_bytes = ctx->deviceBytes;
  int rb = 0;
  cudaStreamSynchronize(ctx->stream);
  cudaMemcpy(&rb, ctx->d.iscal + IS_REBUILDS, sizeof(int), cudaMemcpyDeviceToHost);
  info->neighbour_rebuilds = rb;
  return LBDEM_OK;
}

namespace {
// a download temporary, freed on every return path
struct DeviceTemp {
  double* p = nullptr;
  DeviceTemp() = default;
  DeviceTemp(const DeviceTemp&) = delete;
  DeviceTemp& operator=(const DeviceTemp&) = delete;
  ~DeviceTemp() {
    if (p) cudaFree(p);
  }
};

int d2h(lbdem_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (!dst) return LBDEM_OK;
  CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  return LBDEM_OK;
}
// [3][P] device -> [P][3] host
int d2h3(lbdem_ctx* ctx, double* dst, const double* src, int P) {
  if (!dst) return LBDEM_OK;
  std::vector<double> tmp(3 * (size_t)P);
  CK(cudaMemcpy(tmp.data(), src, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int i = 0; i < P; ++i)
    for (int c = 0; c < 3; ++c) dst[3 * i + c] = tmp[(size_t)c * P + i];
  return LBDEM_OK;
}
}  // namespace

extern "C" int lbdem_download_lattice(lbdem_ctx* ctx, uint8_t* type, uint8_t* pflag,
                                      int32_t* solid, double* n, double* u, double* mass,
                                      double* f) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  int rc = lbdem_sync(ctx);
  if (rc) return rc;
  const size_t N = (size_t)ctx->k.N;
  Device& d = ctx->d;
  if (type || pflag) {
    std::vector<uint8_t> m(N);
    CK(cudaMemcpy(m.data(), d.mask, N, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < N; ++i) {
      if (type) type[i] = m[i] & TYPE_MASK;
      if (pflag) pflag[i] = (m[i] & PFLAG) ? 1 : 0;
    }
  }
  if ((rc = d2h(ctx, solid, d.solid, N * 4))) return rc;
  if (mass || f) {
    DeviceTemp t;
    lbdemNoteDeviceAllocation();
    CK(cudaMalloc(&t.p, (size_t)(Q + 1) * N * sizeof(double)));
    double* tmp = t.p;
    exportLattice<<<latticeGrid(ctx), 256, 0, ctx->stream>>>(ctx->k, d.mask, d.f[ctx->cur], d.mass,
                                                             d.nF, tmp, tmp + (size_t)Q * N);
    CK(cudaStreamSynchronize(ctx->stream));
    if (f) CK(cudaMemcpy(f, tmp, (size_t)Q * N * 8, cudaMemcpyDeviceToHost));
    if (mass) CK(cudaMemcpy(mass, tmp + (size_t)Q * N, N * 8, cudaMemcpyDeviceToHost));
  }
  if (n || u) {
    DeviceTemp t;
    lbdemNoteDeviceAllocation();
    CK(cudaMalloc(&t.p, 4 * N * sizeof(double)));
    double* tmp = t.p;
    momentsKernel<<<latticeGrid(ctx), 256, 0, ctx->stream>>>(ctx->k, d.mask,
                                                             d.f[ctx->cur], tmp,
                                                             tmp + N);
    CK(cudaStreamSynchronize(ctx->stream));
    if (n) CK(cudaMemcpy(n, tmp, N * 8, cudaMemcpyDeviceToHost));
    if (u) CK(cudaMemcpy(u, tmp + N, 3 * N * 8, cudaMemcpyDeviceToHost));
  }
  return LBDEM_OK;
}

extern "C" int lbdem_download_particles(lbdem_ctx* ctx, const lbdem_particle_view* v) {
  if (!ctx || !v) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  int rc = lbdem_sync(ctx);
  if (rc) return rc;
  Device& d = ctx->d;
  const int P = ctx->nPart;
  if (P == 0) return LBDEM_OK;
  const struct { double* dst; const double* src; } m3[] = {
      {v->x0, d.px0},         {v->x1, d.px1},         {v->w1, d.pw1},
      {v->FHydro, d.pFHydro}, {v->MHydro, d.pMHydro}, {v->FContact, d.pFContact},
      {v->MContact, d.pMContact}, {v->FLub, d.pFLub}, {v->MLub, d.pMLub},
      {v->FRep, d.pFRep},     {v->FTotal, d.pFTotal}, {v->MTotal, d.pMTotal},
      {v->xiw, d.pxiw},       {v->xio, d.pxio}};
  for (const auto& e : m3)
    if ((rc = d2h3(ctx, e.dst, e.src, P))) return rc;
  if ((rc = d2h(ctx, v->fluidVolume, d.pFluidVol, (size_t)P * 8))) return rc;
  if (v->SHydro) {
    std::vector<double> tmp(9 * (size_t)P);
    CK(cudaMemcpy(tmp.data(), d.pSHydro, tmp.size() * 8, cudaMemcpyDeviceToHost));
    for (int i = 0; i < P; ++i)
      for (int c = 0; c < 9; ++c) v->SHydro[9 * i + c] = tmp[(size_t)c * P + i];
  }
  int cur = 0;
  CK(cudaMemcpy(&cur, d.iscal + IS_LISTCUR, sizeof(int), cudaMemcpyDeviceToHost));
  if ((rc = d2h(ctx, v->list, d.plist[cur], (size_t)P * MAX_N * 4))) return rc;
  if ((rc = d2h(ctx, v->xi, d.pxi[cur], (size_t)P * 3 * MAX_N * 8))) return rc;
  return LBDEM_OK;
}

extern "C" int lbdem_download_objects(lbdem_ctx* ctx, const lbdem_object_view* v) {
  if (!ctx || !v) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  const int O = ctx->nObj;
  std::vector<double> h((size_t)std::max(O, 1) * OB_STRIDE);
  if (int rc = syncAndRead(ctx, h.data(), ctx->d.obj, h.size() * 8)) return rc;
  const struct { double* dst; int off; } m[] = {
      {v->x0, OB_X0},       {v->x1, OB_X1},       {v->w1, OB_W1},
      {v->FHydro, OB_FHYDRO}, {v->MHydro, OB_MHYDRO}, {v->FContact, OB_FCONTACT},
      {v->MContact, OB_MCONTACT}, {v->FLub, OB_FLUB}, {v->MLub, OB_MLUB},
      {v->FTotal, OB_FTOTAL}};
  for (const auto& e : m)
    if (e.dst)
      for (int o = 0; o < O; ++o)
        for (int c = 0; c < 3; ++c) e.dst[3 * o + c] = h[(size_t)o * OB_STRIDE + e.off + c];
  return LBDEM_OK;
}

extern "C" int lbdem_download_bodies(lbdem_ctx* ctx, double* x0, double* x1, double* FSpring,
                                     double* FTotal, double* L) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  const int B = ctx->nBody;
  if (B == 0) return lbdem_sync(ctx);
  std::vector<double> h((size_t)B * BD_STRIDE);
  if (int rc = syncAndRead(ctx, h.data(), ctx->d.body, h.size() * 8)) return rc;
  const struct { double* dst; int off; } m[] = {
      {x0, BD_X0}, {x1, BD_X1}, {FSpring, BD_FSPRING}, {FTotal, BD_FTOTAL}};
  for (const auto& e : m)
    if (e.dst)
      for (int b = 0; b < B; ++b)
        for (int q = 0; q < 3; ++q) e.dst[3 * b + q] = h[(size_t)b * BD_STRIDE + e.off + q];
  if (L)
    for (int b = 0; b < B; ++b) L[b] = h[(size_t)b * BD_STRIDE + BD_L];
  return LBDEM_OK;
}

extern "C" int lbdem_download_viscosity(lbdem_ctx* ctx, double* visc) {
  if (!ctx || !visc) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  int rc = lbdem_sync(ctx);
  if (rc) return rc;
  const size_t N = (size_t)ctx->k.N;
  std::vector<uint8_t> m(N);
  CK(cudaMemcpy(m.data(), ctx->d.mask, N, cudaMemcpyDeviceToHost));
  if (ctx->d.visc) CK(cudaMemcpy(visc, ctx->d.visc, N * sizeof(double), cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < N; ++i) {
    if (!isActiveT(m[i] & TYPE_MASK)) visc[i] = 0.0;
    else if (!ctx->d.visc) visc[i] = ctx->k.initVisc;
  }
  return LBDEM_OK;
}

extern "C" int lbdem_download_walls(lbdem_ctx* ctx, double* FHydro, double* FContact,
                                    double* FLub, double* FTotal) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  int rc = lbdem_sync(ctx);
  if (rc) return rc;
  const int W = ctx->nWall;
  std::vector<double> h((size_t)MAX_WALL * 12);
  CK(cudaMemcpy(h.data(), ctx->d.wallF, h.size() * 8, cudaMemcpyDeviceToHost));
  double* outs[4] = {FHydro, FContact, FLub, FTotal};
  for (int q = 0; q < 4; ++q)
    if (outs[q])
      for (int w = 0; w < W; ++w)
        for (int c = 0; c < 3; ++c) outs[q][3 * w + c] = h[(size_t)w * 12 + 3 * q + c];
  return LBDEM_OK;
}

namespace {
int massSums(lbdem_ctx* ctx, int withParticles, double* total_mass, int64_t* interface_nodes,
             int64_t* active_nodes) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  int rc = lbdem_sync(ctx);
  if (rc) return rc;
  // stream-ordered temporary: no device-wide synchronisation
  double* tmp = nullptr;
  lbdemNoteDeviceAllocation();
  CK(cudaMallocAsync(&tmp, 3 * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(tmp, 0, 3 * sizeof(double), ctx->stream));
  massSummaryKernel<<<latticeGrid(ctx), 256, 0, ctx->stream>>>(
      ctx->k, ctx->d.mask, ctx->d.mass, ctx->d.nF, tmp, (unsigned long long*)(tmp + 1), withParticles);
  double m = 0;
  unsigned long long c[2] = {0, 0};
  CK(cudaMemcpyAsync(&m, tmp, 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(c, tmp + 1, 16, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaFreeAsync(tmp, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (total_mass) *total_mass = m;
  if (interface_nodes) *interface_nodes = (int64_t)c[0];
  if (active_nodes) *active_nodes = (int64_t)c[1];
  return LBDEM_OK;
}
}  // namespace

extern "C" int lbdem_mass_summary(lbdem_ctx* ctx, double* total_mass,
                                  int64_t* interface_nodes, int64_t* active_nodes) {
  return massSums(ctx, 0, total_mass, interface_nodes, active_nodes);
}

extern "C" int lbdem_mass_total(lbdem_ctx* ctx, double* total_mass) {
  return massSums(ctx, 1, total_mass, nullptr, nullptr);
}
