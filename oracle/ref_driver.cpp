// Driver for the pinned reference build (TEST INFRASTRUCTURE ONLY).
//
// Links the reference's own, unmodified LB/DEM sources (compiled straight
// from the reference tree by oracle/Makefile) and replays the reference
// time loop:
//   init sequence   = src/main.cpp:239-286 (parseConfigFile, latticeDefinition,
//                     discreteElementInit, latticeBolzmannInit, time reset)
//   one step        = goCycle, src/main.cpp:38-67; IO::outputStep only with
//                     -io DIR (the reference's own IO code, src/IO.cpp, with
//                     every VTK export time 0: the screen-phase files
//                     export.dat, objPosition.dat, objForce.dat,
//                     wallForce.dat and the stress files, in DIR, the
//                     fluid recycle files in DIR/fluidData at
//                     fluidRecycleExpTime and the particle recycle files in
//                     DIR/particleData at partRecycleExpTime)
// Defined-behaviour pins applied here, at the public-member level, without
// touching the reference sources:
//   * particle::list/_list/xix/xiy/xiz/_xix/_xiy/_xiz (src/elmt.h:44-51) are
//     left uninitialised by the particle constructor (src/elmt.h:100-127);
//     they are zeroed right after DEM::discreteElementGet, which only copies
//     constructed particles into DEM::particles (src/DEM.cpp:88-134).
//   * uninitialised locals (src/DEM.cpp:916,1950,2161,2771) are zeroed by
//     compiling with -ftrivial-auto-var-init=zero (oracle/Makefile).
//   * no OpenMP, -ffp-contract=off: serial, FMA-free, identical on x86/Arm.
// Output: full-precision state dumps (oracle/statedump.h) and a timing line.
//
// usage: lbdem_ref -c parameters.cfg -steps N [-dump DIR] [-every K]
//                  [-io DIR] [-time] [-anyReferenceKey value ...]
// Inputs particles.dat / objects.dat / body.dat are read from ./input/ under
// the working directory, exactly as the reference does (src/DEM.cpp:81,138,169).
#include <sys/stat.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "DEM.h"
#include "IO.h"
#include "LB.h"
#include "getpot.h"
#include "statedump.h"

ProblemName problemName = NONE;

namespace {

struct RunFlags {
  bool demSolve = false, lbSolve = false;
};

void dumpState(const std::string& path, int step, LB& lb, DEM& dem) {
  lbdump::Writer w(path);
  w.scalari("step", step);
  w.scalar("demTime", dem.demTime);
  w.scalari("demTimeStep", dem.demTimeStep);
  const size_t N = lb.totNodes;
  if (N) {
    std::vector<int32_t> size = {(int32_t)lb.lbSize[0], (int32_t)lb.lbSize[1],
                                 (int32_t)lb.lbSize[2]};
    w.i("lbSize", size);
    std::vector<uint8_t> type(N), pflag(N), hasnode(N);
    std::vector<int32_t> solid(N);
    std::vector<double> n(N, 0.0), ux(N, 0.0), uy(N, 0.0), uz(N, 0.0),
        mass(N, 0.0), visc(N, 0.0), f(19 * N, 0.0);
    for (size_t it = 0; it < N; ++it) {
      type[it] = (uint8_t)lb.types[it].getType();
      pflag[it] = lb.types[it].isInsideParticle() ? 1 : 0;
      solid[it] = (int32_t)lb.types[it].getSolidIndex();
      const node* nd = lb.nodes[it];
      hasnode[it] = nd ? 1 : 0;
      if (nd && lb.types[it].isActive()) {
        n[it] = nd->n;
        ux[it] = nd->u.x;
        uy[it] = nd->u.y;
        uz[it] = nd->u.z;
        mass[it] = nd->mass;
        visc[it] = nd->visc;
        for (int j = 0; j < 19; ++j) f[(size_t)j * N + it] = nd->f[j];
      }
    }
    w.b("type", type);
    w.b("pflag", pflag);
    w.b("hasnode", hasnode);
    w.i("solid", solid);
    w.d("n", n);
    w.d("ux", ux);
    w.d("uy", uy);
    w.d("uz", uz);
    w.d("mass", mass);
    w.d("visc", visc);
    w.d("f", f, {19, N});
  }
  const size_t P = dem.particles.size();
  std::vector<double> pv;
  auto vec3 = [&](const char* name, auto get) {
    pv.assign(3 * P, 0.0);
    for (size_t i = 0; i < P; ++i) {
      const tVect v = get(dem.particles[i]);
      pv[3 * i] = v.x;
      pv[3 * i + 1] = v.y;
      pv[3 * i + 2] = v.z;
    }
    w.d(name, pv, {P, 3});
  };
  vec3("p_x0", [](const particle& p) { return p.x0; });
  vec3("p_x1", [](const particle& p) { return p.x1; });
  vec3("p_w1", [](const particle& p) { return p.w1; });
  vec3("p_FHydro", [](const particle& p) { return p.FHydro; });
  vec3("p_MHydro", [](const particle& p) { return p.MHydro; });
  vec3("p_FContact", [](const particle& p) { return p.FContact; });
  vec3("p_MContact", [](const particle& p) { return p.MContact; });
  vec3("p_FLub", [](const particle& p) { return p.FLub; });
  vec3("p_MLub", [](const particle& p) { return p.MLub; });
  vec3("p_FRep", [](const particle& p) { return p.FRep; });
  vec3("p_FTotal", [](const particle& p) { return p.FTotal; });
  vec3("p_MTotal", [](const particle& p) { return p.MTotal; });
  vec3("p_FGrav", [](const particle& p) { return p.FGrav; });
  vec3("p_xiw", [](const particle& p) { return p.xiw; });
  vec3("p_xio", [](const particle& p) { return p.xio; });
  {
    std::vector<double> fv(P), s(9 * P);
    for (size_t i = 0; i < P; ++i) {
      fv[i] = dem.particles[i].fluidVolume;
      const tMat& m = dem.particles[i].SHydro;
      const double a[9] = {m.m00, m.m01, m.m02, m.m10, m.m11,
                           m.m12, m.m20, m.m21, m.m22};
      for (int k = 0; k < 9; ++k) s[9 * i + k] = a[k];
    }
    w.d("p_fluidVolume", fv);
    w.d("p_SHydro", s, {P, 9});
    std::vector<int32_t> lst(50 * P);
    std::vector<double> xi(3 * 50 * P);
    for (size_t i = 0; i < P; ++i)
      for (int k = 0; k < 50; ++k) {
        lst[50 * i + k] = dem.particles[i].list[k];
        xi[150 * i + k] = dem.particles[i].xix[k];
        xi[150 * i + 50 + k] = dem.particles[i].xiy[k];
        xi[150 * i + 100 + k] = dem.particles[i].xiz[k];
      }
    w.i("p_list", lst, {P, 50});
    w.d("p_xi", xi, {P, 3, 50});
  }
  const size_t O = dem.objects.size();
  std::vector<double> ov(O * 3);
  auto ovec = [&](const char* name, auto get) {
    for (size_t o = 0; o < O; ++o) {
      const tVect v = get(dem.objects[o]);
      ov[3 * o] = v.x;
      ov[3 * o + 1] = v.y;
      ov[3 * o + 2] = v.z;
    }
    w.d(name, ov, {O, 3});
  };
  ovec("o_x0", [](const object& o) { return o.x0; });
  ovec("o_x1", [](const object& o) { return o.x1; });
  ovec("o_w1", [](const object& o) { return o.w1; });
  ovec("o_FHydro", [](const object& o) { return o.FHydro; });
  ovec("o_MHydro", [](const object& o) { return o.MHydro; });
  ovec("o_FContact", [](const object& o) { return o.FContact; });
  ovec("o_MContact", [](const object& o) { return o.MContact; });
  ovec("o_FLub", [](const object& o) { return o.FLub; });
  ovec("o_MLub", [](const object& o) { return o.MLub; });
  ovec("o_FTotal", [](const object& o) { return o.FTotal; });
  const size_t W = dem.walls.size();
  std::vector<double> wv(W * 3);
  auto wvec = [&](const char* name, auto get) {
    for (size_t k = 0; k < W; ++k) {
      const tVect v = get(dem.walls[k]);
      wv[3 * k] = v.x;
      wv[3 * k + 1] = v.y;
      wv[3 * k + 2] = v.z;
    }
    w.d(name, wv, {W, 3});
  };
  wvec("w_FHydro", [](const wall& x) { return x.FHydro; });
  wvec("w_FContact", [](const wall& x) { return x.FContact; });
  wvec("w_FLub", [](const wall& x) { return x.FLub; });
  wvec("w_FTotal", [](const wall& x) { return x.FTotal; });
  const size_t B = dem.bodies.size();
  if (B) {
    std::vector<double> bv(B * 3), bl(B);
    auto bvec = [&](const char* name, auto get) {
      for (size_t b = 0; b < B; ++b) {
        const tVect v = get(dem.bodies[b]);
        bv[3 * b] = v.x;
        bv[3 * b + 1] = v.y;
        bv[3 * b + 2] = v.z;
      }
      w.d(name, bv, {B, 3});
    };
    bvec("b_x0", [](const body& b) { return b.x0; });
    bvec("b_x1", [](const body& b) { return b.x1; });
    bvec("b_FSpring", [](const body& b) { return b.FSpring; });
    bvec("b_FTotal", [](const body& b) { return b.FTotal; });
    for (size_t b = 0; b < B; ++b) bl[b] = dem.bodies[b].L;
    w.d("b_L", bl);
  }
  w.close();
}

}  // namespace

int main(int argc, char** argv) {
  GetPot commandLine(argc, argv);
  std::string cfg = "config.cfg";
  if (commandLine.search("-c")) cfg = commandLine.next(cfg.c_str());
  int steps = 0;
  if (commandLine.search("-steps")) steps = commandLine.next(0);
  std::string dumpDir;
  if (commandLine.search("-dump")) dumpDir = commandLine.next("");
  int every = 1;
  if (commandLine.search("-every")) every = commandLine.next(1);
  const bool timing = commandLine.search("-time");
  std::string ioDir;
  if (commandLine.search("-io")) ioDir = commandLine.next("");

  GetPot configFile(cfg.c_str());
  DEM dem;
  LB lb;
  RunFlags run;
  // src/main.cpp:128-185 (parseConfigFile): only the keys the step reads.
  PARSE_CLASS_MEMBER(configFile, dem.demInitialRepeat, "demInitialRepeat", 0.0);
  PARSE_CLASS_MEMBER(configFile, lb.lbmInitialRepeat, "lbmInitialRepeat", 0);
  PARSE_CLASS_MEMBER(configFile, run.demSolve, "demSolve", 0);
  PARSE_CLASS_MEMBER(configFile, run.lbSolve, "lbSolve", 0);
  PARSE_CLASS_MEMBER(configFile, lb.freeSurface, "freeSurfaceSolve", 0);
  PARSE_CLASS_MEMBER(configFile, lb.forceField, "forceFieldSolve", 0);
  lb.latticeBoltzmannGet(configFile, commandLine);
  dem.discreteElementGet(configFile, commandLine);

  // Pin (1): zero the neighbour-list and tangential-history arrays.
  for (size_t i = 0; i < dem.particles.size(); ++i) {
    particle& p = dem.particles[i];
    std::memset(p.list, 0, sizeof(p.list));
    std::memset(p._list, 0, sizeof(p._list));
    std::memset(p.xix, 0, sizeof(p.xix));
    std::memset(p.xiy, 0, sizeof(p.xiy));
    std::memset(p.xiz, 0, sizeof(p.xiz));
    std::memset(p._xix, 0, sizeof(p._xix));
    std::memset(p._xiy, 0, sizeof(p._xiy));
    std::memset(p._xiz, 0, sizeof(p._xiz));
  }

  // src/main.cpp:264-283
  lb.latticeDefinition();
  const tVect externalForce = lb.lbF * lb.unit.Accel;
  dem.discreteElementInit(lb.boundary, lb.lbPhysicalSize, lb.lbBoundaryLocation,
                          lb.unit.Time, externalForce, lb.fluidHeight,
                          lb.freeSurface);
  if (run.lbSolve) lb.latticeBolzmannInit(dem.walls, dem.particles, dem.objects);
  lb.time = 0;
  dem.demTime = 0.0;
  dem.demTimeStep = 0;

  // IO as src/main.cpp:75-120, 128-185 and 282-286 set it up, screen phase only
  IO io;
  if (!ioDir.empty()) {
    io.workDirectory = ioDir;
    ::mkdir(ioDir.c_str(), 0777);
    io.demSolve = run.demSolve;
    io.lbmSolve = run.lbSolve;
    PARSE_CLASS_MEMBER(configFile, io.screenExpTime, "screenExpTime", 0.0);
    io.stateExpTime = io.fluidExpTime = io.fluidLagrangianExpTime = io.fluid2DExpTime = 0.0;
    io.partExpTime = io.boundExpTime = io.objectExpTime = io.bodyExpTime = 0.0;
    io.springExpTime = io.objectExpTime2 = io.chainExpTime = io.velExpTime = 0.0;
    io.dispExpTime = io.stressExpTime = io.part_yDispExpTime = io.part_rDispExpTime = 0.0;
    io.part_n1ExpTime = io.part_n2ExpTime = io.part_pressureExpTime = 0.0;
    io.part_yyStressExpTime = 0.0;
    PARSE_CLASS_MEMBER(configFile, io.partRecycleExpTime, "partRecycleExpTime", 0.0);
    PARSE_CLASS_MEMBER(configFile, io.fluidRecycleExpTime, "fluidRecycleExpTime", 0.0);
    io.outputExpTime = io.simComplexExpTime = 0.0;
    io.initialize();
    io.currentTimeStep = 0;
    io.realTime = 0.0;
    io.outputStep(lb, dem);
  }

  auto dumpName = [&](int s) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "/dump_%06d.bin", s);
    return dumpDir + buf;
  };
  if (!dumpDir.empty()) {
    ::mkdir(dumpDir.c_str(), 0777);
    dumpState(dumpName(0), 0, lb, dem);
  }

  double seconds = 0.0;
  for (int s = 1; s <= steps; ++s) {
    const auto t0 = std::chrono::steady_clock::now();
    // goCycle, src/main.cpp:38-67
    io.realTime += lb.unit.Time;
    ++io.currentTimeStep;
    ++lb.time;
    if (run.demSolve) dem.discreteElementStep(lb.boundary);
    if (run.lbSolve && dem.demTime >= dem.demInitialRepeat) {
      if (run.demSolve)
        lb.latticeBoltzmannCouplingStep(dem.newNeighborList, dem.particles,
                                        dem.objects);
      lb.latticeBolzmannStep(dem.particles, dem.walls, dem.objects);
      if (lb.freeSurface) lb.latticeBoltzmannFreeSurfaceStep();
    } else if (run.lbSolve && dem.demTime <= dem.demInitialRepeat) {
      if (run.demSolve)
        lb.latticeBoltzmannCouplingStep(dem.newNeighborList, dem.particles,
                                        dem.objects);
    }
    const auto t1 = std::chrono::steady_clock::now();
    seconds += std::chrono::duration<double>(t1 - t0).count();
    if (!ioDir.empty()) io.outputStep(lb, dem);
    if (!dumpDir.empty() && (s % every == 0 || s == steps))
      dumpState(dumpName(s), s, lb, dem);
  }
  if (timing) {
    size_t active = 0;
    for (size_t it = 0; it < lb.totNodes; ++it)
      if (lb.types[it].isActive()) ++active;
    std::printf(
        "{\"steps\": %d, \"seconds\": %.6f, \"ms_per_step\": %.3f, "
        "\"active_nodes\": %zu, \"nodes\": %u, \"particles\": %zu}\n",
        steps, seconds, steps ? 1e3 * seconds / steps : 0.0, active,
        lb.totNodes, dem.particles.size());
  }
  return 0;
}
