// The reference's screen-phase output files, written from the run's device
// state without synchronising its stream.
//
// Reference: IO::initialize (src/IO.cpp:8-94) creates the files and their
// header lines; IO::outputStep (src/IO.cpp:113-158) runs once before the
// first goCycle and after every goCycle (src/main.cpp:66, 286), and when
// the screen counter (unsigned)(realTime / screenExpTime) + 1 has advanced
// it appends one line to export.dat and, with the DEM on, the impactor
// lines (IO::exportObjectPosition / exportObjectForce, src/IO.cpp:1239-1353)
// and the wall line (IO::exportWallForce, src/IO.cpp:1295-1314). realTime is
// the sum of unitTime over the cycles, added one cycle at a time as goCycle
// does, so the same cycles are picked. Numbers are printed as the
// reference's streams print them: six significant digits ("%g"), each
// vector as "x y z ", groups separated by tabs.
//
// At an output cycle the impactor records and the wall-force records are
// copied on the run's stream into a slot of a pinned ring, followed by an
// event; the lines are formatted once the event has completed (checked
// after each lbdem_cycle call, waited for by lbdem_sync and
// lbdem_output_close). A full ring waits for its oldest slot.
//
// With lbdem_output_recycle the recycle files of IO::createFiles
// (src/IO.cpp:201-210, 268-274) are written as well: dir/fluidData/
// fluidRecycle%010u.dat, named by the cycle, whenever the counter
// (unsigned)(realTime / fluidRecycleExpTime) + 1 advances, and
// dir/particleData/partRecycle%04u.dat, named by its counter, whenever the
// partRecycleExpTime counter does (both at the first cycle too).
// IO::exportRecycleParticles (src/IO.cpp:999-1030) writes per particle the
// radius, position and velocity, then the negated total stresslet (xx, yy,
// zz and the three mean off-diagonal pairs) and the negated vertical
// displacement since the start, tab-separated. Each file synchronises the
// stream.
//
// The stress files (IO::exportStressTensor and the two contribution files,
// src/IO.cpp:1355-1409) take the DEM stress sums of the cycle's DEM step
// (demStress, launched on the cycles whose line is due), each divided by
// the DEM volume: the total as xx yy zz and the mean off-diagonal pairs
// (tinyMatrix::print, src/myvector.cpp:382-392), the hydrodynamic,
// lubrication, contact and electrostatic parts as their normal and shear
// triples. bodyPosition.dat gets one line per body (IO::exportBodyPosition,
// src/IO.cpp:1340-1352: position, tab, velocity, tab, spring length L) after
// the impactor lines of a run with bodies, and only its header otherwise.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "kernels_decl.h"
#include "lbdem_internal.h"

using namespace lbdem;

struct lbdem_output {
  std::string dir;
  double screenExp = 0.0, unitTime = 0.0, fluidHeight = 0.0;
  double realTime = 0.0;   // IO::realTime
  unsigned lastScreen = 0; // IO::lastScreenExp
  double recycleExp = 0.0;  // IO::fluidRecycleExpTime (0: off)
  unsigned lastRecycle = 0; // IO::lastFluidRecycleExp
  double partExp = 0.0;     // IO::partRecycleExpTime (0: off)
  unsigned lastPart = 0;    // IO::lastPartRecycleExp
  bool dem = false;
  std::FILE* fExport = nullptr;
  std::FILE* fPos = nullptr;
  std::FILE* fBody = nullptr;  // bodyPosition.dat, open while the run has bodies
  int nBody = 0;
  std::FILE* fForce = nullptr;
  std::FILE* fWall = nullptr;
  std::FILE* fStress = nullptr;
  std::FILE* fNormal = nullptr;
  std::FILE* fShear = nullptr;
  double vol = 1.0;  // DEM::vol, src/DEM.cpp:211-215
  int nObj = 0, nWall = 0;
  size_t slotDoubles = 0;  // nObj * OB_STRIDE + nWall * 12 + STRESS_N
  double* pinned = nullptr;
  struct Slot {
    cudaEvent_t ev = nullptr;
    unsigned long long step = 0;
    double realTime = 0.0;
  };
  std::vector<Slot> slots;
  size_t head = 0, count = 0;  // FIFO of slots whose copy is in flight
};

namespace {

constexpr int kSlots = 64;

int fail(lbdem_ctx* ctx, int code, const std::string& msg) {
  ctx->err = msg;
  return code;
}

unsigned screenCounter(const lbdem_output* o, double t) {
  return o->screenExp > 0.0 ? static_cast<unsigned>(t / o->screenExp) + 1u : 0u;
}
unsigned recycleCounter(const lbdem_output* o, double t) {
  return o->recycleExp > 0.0 ? static_cast<unsigned>(t / o->recycleExp) + 1u : 0u;
}
unsigned partCounter(const lbdem_output* o, double t) {
  return o->partExp > 0.0 ? static_cast<unsigned>(t / o->partExp) + 1u : 0u;
}

// IO::exportRecycleParticles, named by the counter (waits for the run's work)
int writePartRecycle(lbdem_ctx* ctx, unsigned counter) {
  int rc = lbdem_sync(ctx);
  if (rc) return rc;
  const int P = ctx->nPart;
  std::vector<double> r(P), x0(3 * (size_t)P), x1(3 * (size_t)P), S(9 * (size_t)P), dy(P);
  const Device& d = ctx->d;
  cudaError_t e = cudaSuccess;
  if (P > 0) {
    e = cudaMemcpy(r.data(), d.pr, P * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(x0.data(), d.px0, 3 * P * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(x1.data(), d.px1, 3 * P * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(S.data(), d.pStress, 9 * P * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(dy.data(), d.dispY, P * sizeof(double), cudaMemcpyDeviceToHost);
  }
  if (e != cudaSuccess)
    return fail(ctx, LBDEM_ERR_CUDA, std::string("particle recycle: ") + cudaGetErrorString(e));
  char name[64];
  std::snprintf(name, sizeof name, "/particleData/partRecycle%04u.dat", counter);
  std::FILE* f = std::fopen((ctx->out->dir + name).c_str(), "w");
  if (!f) return fail(ctx, LBDEM_ERR_IO, std::string("cannot write ") + ctx->out->dir + name);
  for (int i = 0; i < P; ++i) {
    auto m = [&](int c) { return S[(size_t)c * P + i]; };
    std::fprintf(f, "%g ", r[i]);
    std::fprintf(f, "%g %g %g ", x0[i], x0[P + i], x0[2 * (size_t)P + i]);
    std::fprintf(f, "%g %g %g ", x1[i], x1[P + i], x1[2 * (size_t)P + i]);
    std::fprintf(f, "%g\t%g\t%g\t%g\t%g\t%g\t%g\n", -m(0), -m(4), -m(8), -(m(1) + m(3)) * 0.5,
                 -(m(5) + m(7)) * 0.5, -(m(2) + m(6)) * 0.5, -dy[i]);
  }
  if (std::fclose(f) != 0) return fail(ctx, LBDEM_ERR_IO, std::string("write failed: ") + name);
  return LBDEM_OK;
}

// IO::exportRecycleFluid at this cycle (waits for the run's work)
int writeRecycle(lbdem_ctx* ctx) {
  char name[64];
  std::snprintf(name, sizeof name, "/fluidData/fluidRecycle%010u.dat", (unsigned)ctx->lbTime);
  return lbdem_export_recycle_fluid(ctx, (ctx->out->dir + name).c_str());
}

void vec(std::FILE* f, const double* v) { std::fprintf(f, "%g %g %g ", v[0], v[1], v[2]); }
// tinyMatrix::printNormal / printShear of a row-major 3x3
void normal3(std::FILE* f, const double* m) { std::fprintf(f, "%g %g %g ", m[0], m[4], m[8]); }
void shear3(std::FILE* f, const double* m) {
  std::fprintf(f, "%g %g %g ", (m[1] + m[3]) / 2.0, (m[5] + m[7]) / 2.0, (m[2] + m[6]) / 2.0);
}

// the lines of one captured cycle
void writeSlot(lbdem_output* o, const lbdem_output::Slot& s, const double* rec) {
  std::fprintf(o->fExport, "%llu; time=%g\t\n", s.step, s.realTime);
  if (o->dem && o->nObj > 0) {
    for (int i = 0; i < o->nObj; ++i) {
      const double* ob = rec + (size_t)i * OB_STRIDE;
      const double r = ob[OB_R];
      const double depth = (o->fluidHeight + r) - ob[OB_X0 + 1];
      vec(o->fPos, ob + OB_X0);
      std::fputs("\t", o->fPos);
      vec(o->fPos, ob + OB_X1);
      std::fprintf(o->fPos, "\t%g\n", depth);
    }
    for (int i = 0; i < o->nObj; ++i) {
      const double* ob = rec + (size_t)i * OB_STRIDE;
      const double r = ob[OB_R];
      const double depth = (o->fluidHeight + r) - ob[OB_X0 + 1];
      double fe[3], se[3] = {0.0, 0.0, 0.0};
      for (int c = 0; c < 3; ++c) fe[c] = ob[OB_FTOTAL + c] - ob[OB_FGRAV + c];
      if (depth > 0) {
        const double area = 4.0 * M_PI * r * r * (depth / (2.0 * r));
        for (int c = 0; c < 3; ++c) se[c] = fe[c] / area;
      }
      const double zero[3] = {0.0, 0.0, 0.0};  // an impactor's FRep is never set
      const double* groups[7] = {fe, se, ob + OB_FTOTAL, ob + OB_FCONTACT, ob + OB_FHYDRO,
                                 ob + OB_FLUB, zero};
      for (int g = 0; g < 7; ++g) {
        vec(o->fForce, groups[g]);
        std::fputs(g < 6 ? "\t" : "\n", o->fForce);
      }
    }
  }
  if (o->dem && o->nBody > 0) {
    const double* bd0 = rec + (size_t)o->nObj * OB_STRIDE + (size_t)o->nWall * 12 + STRESS_N;
    for (int b = 0; b < o->nBody; ++b) {
      const double* bd = bd0 + (size_t)b * BD_STRIDE;
      vec(o->fBody, bd + BD_X0);
      std::fputs("\t", o->fBody);
      vec(o->fBody, bd + BD_X1);
      std::fprintf(o->fBody, "\t%g\n", bd[BD_L]);
    }
  }
  if (o->dem && o->nWall > 0) {
    const double* wf = rec + (size_t)o->nObj * OB_STRIDE;
    for (int w = 0; w < o->nWall; ++w) {
      vec(o->fWall, wf + 12 * w + 9);  // FTotal
      std::fputs("\t", o->fWall);
      vec(o->fWall, wf + 12 * w + 3);  // FContact
      std::fputs("\t", o->fWall);
    }
    std::fputs("\n", o->fWall);
  }
  if (o->dem) {
    // DEM::evaluateForces: each part over the volume, then the total
    const double* raw = rec + (size_t)o->nObj * OB_STRIDE + (size_t)o->nWall * 12;
    double part[4][9], total[9];
    for (int p = 0; p < 4; ++p)
      for (int c = 0; c < 9; ++c) part[p][c] = raw[9 * p + c] / o->vol;
    const double* contact = part[0];
    const double* lub = part[1];
    const double* electro = part[2];
    const double* hydro = part[3];
    for (int c = 0; c < 9; ++c) total[c] = 0.0 + (((contact[c] + lub[c]) + electro[c]) + hydro[c]);
    normal3(o->fStress, total);
    shear3(o->fStress, total);
    std::fputs("\n", o->fStress);
    const double* order[4] = {hydro, lub, contact, electro};
    for (int p = 0; p < 4; ++p) {
      normal3(o->fNormal, order[p]);
      std::fputs(p < 3 ? "\t" : "\n", o->fNormal);
      shear3(o->fShear, order[p]);
      std::fputs(p < 3 ? "\t" : "\n", o->fShear);
    }
  }
}

// writes the oldest pending slot; waits for its copy if `wait`
int writeOldest(lbdem_ctx* ctx, bool wait, bool* wrote) {
  lbdem_output* o = ctx->out;
  *wrote = false;
  if (!o->count) return LBDEM_OK;
  lbdem_output::Slot& s = o->slots[o->head];
  cudaError_t e = wait ? cudaEventSynchronize(s.ev) : cudaEventQuery(s.ev);
  if (e == cudaErrorNotReady) return LBDEM_OK;
  if (e != cudaSuccess)
    return fail(ctx, LBDEM_ERR_CUDA, std::string("output copy: ") + cudaGetErrorString(e));
  writeSlot(o, s, o->pinned + o->head * o->slotDoubles);
  o->head = (o->head + 1) % o->slots.size();
  --o->count;
  *wrote = true;
  return LBDEM_OK;
}

// enqueues the copy of this cycle's impactor and wall records
int capture(lbdem_ctx* ctx) {
  lbdem_output* o = ctx->out;
  bool wrote = false;
  int rc;
  if (o->count == o->slots.size() && (rc = writeOldest(ctx, true, &wrote))) return rc;
  const size_t k = (o->head + o->count) % o->slots.size();
  double* dst = o->pinned + k * o->slotDoubles;
  cudaError_t e = cudaSuccess;
  if (o->nObj > 0)
    e = cudaMemcpyAsync(dst, ctx->d.obj, (size_t)o->nObj * OB_STRIDE * sizeof(double),
                        cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && o->nWall > 0)
    e = cudaMemcpyAsync(dst + (size_t)o->nObj * OB_STRIDE, ctx->d.wallF,
                        (size_t)o->nWall * 12 * sizeof(double), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess && o->dem)
    e = cudaMemcpyAsync(dst + (size_t)o->nObj * OB_STRIDE + (size_t)o->nWall * 12,
                        ctx->d.stress, STRESS_N * sizeof(double), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess && o->dem && o->nBody > 0)
    e = cudaMemcpyAsync(dst + (size_t)o->nObj * OB_STRIDE + (size_t)o->nWall * 12 + STRESS_N,
                        ctx->d.body, (size_t)o->nBody * BD_STRIDE * sizeof(double),
                        cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(o->slots[k].ev, ctx->stream);
  if (e != cudaSuccess)
    return fail(ctx, LBDEM_ERR_CUDA, std::string("output copy: ") + cudaGetErrorString(e));
  o->slots[k].step = (unsigned long long)ctx->lbTime;
  o->slots[k].realTime = o->realTime;
  ++o->count;
  return LBDEM_OK;
}

std::FILE* openWithHeader(const std::string& path, const char* header) {
  std::FILE* f = std::fopen(path.c_str(), "a");
  if (f && header) std::fputs(header, f);
  return f;
}

}  // namespace

bool lbdemOutputDueNext(const lbdem_ctx* ctx) {
  const lbdem_output* o = ctx->out;
  if (!o) return false;
  const double t = o->realTime + o->unitTime;
  return screenCounter(o, t) > o->lastScreen || recycleCounter(o, t) > o->lastRecycle ||
         partCounter(o, t) > o->lastPart;
}

bool lbdemOutputParticleStressNext(const lbdem_ctx* ctx) {
  const lbdem_output* o = ctx->out;
  return o && o->dem && partCounter(o, o->realTime + o->unitTime) > o->lastPart;
}

bool lbdemOutputStressNext(const lbdem_ctx* ctx) {
  const lbdem_output* o = ctx->out;
  return o && o->dem && (screenCounter(o, o->realTime + o->unitTime) > o->lastScreen ||
                         partCounter(o, o->realTime + o->unitTime) > o->lastPart);
}

bool lbdemOutputBlocksPair(const lbdem_ctx* ctx) {
  const lbdem_output* o = ctx->out;
  if (!o) return false;
  if (lbdemOutputDueNext(ctx)) return true;
  const double t2 = (o->realTime + o->unitTime) + o->unitTime;
  return o->dem && (screenCounter(o, t2) > o->lastScreen || partCounter(o, t2) > o->lastPart);
}

int lbdemOutputAfterCycle(lbdem_ctx* ctx) {
  lbdem_output* o = ctx->out;
  if (!o) return LBDEM_OK;
  o->realTime += o->unitTime;
  const unsigned c = screenCounter(o, o->realTime);
  if (c > o->lastScreen) {
    o->lastScreen = c;
    if (int rc = capture(ctx)) return rc;
  }
  const unsigned r = recycleCounter(o, o->realTime);
  if (r > o->lastRecycle) {
    o->lastRecycle = r;
    if (int rc = writeRecycle(ctx)) return rc;
  }
  const unsigned p = partCounter(o, o->realTime);
  if (p > o->lastPart) {
    o->lastPart = p;
    return writePartRecycle(ctx, p);
  }
  return LBDEM_OK;
}

int lbdemOutputDrain(lbdem_ctx* ctx, bool wait) {
  if (!ctx->out) return LBDEM_OK;
  bool wrote = true;
  while (wrote) {
    const int rc = writeOldest(ctx, wait, &wrote);
    if (rc) return rc;
  }
  std::fflush(ctx->out->fExport);
  return LBDEM_OK;
}

void lbdemOutputResync(lbdem_ctx* ctx) {
  lbdem_output* o = ctx->out;
  if (!o) return;
  o->realTime = 0.0;
  for (long long i = 0; i < ctx->lbTime; ++i) o->realTime += o->unitTime;
  o->lastScreen = screenCounter(o, o->realTime);
  o->lastRecycle = recycleCounter(o, o->realTime);
  o->lastPart = partCounter(o, o->realTime);
}

void lbdemOutputFree(lbdem_ctx* ctx) {
  lbdem_output* o = ctx->out;
  if (!o) return;
  for (auto& s : o->slots)
    if (s.ev) cudaEventDestroy(s.ev);
  if (o->pinned) cudaFreeHost(o->pinned);
  for (std::FILE* f : {o->fExport, o->fPos, o->fBody, o->fForce, o->fWall, o->fStress,
                       o->fNormal, o->fShear})
    if (f) std::fclose(f);
  delete o;
  ctx->out = nullptr;
}

extern "C" int lbdem_output_open(lbdem_ctx* ctx, const char* dir, double screen_exp_time) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  if (!dir || !(screen_exp_time >= 0.0))
    return fail(ctx, LBDEM_ERR_INVALID, "output_open: null directory or negative screenExpTime");
  if (ctx->out) return fail(ctx, LBDEM_ERR_INVALID, "output_open: output already open");
  lbdem_output* o = new lbdem_output;
  ctx->out = o;
  o->dir = dir;
  o->screenExp = screen_exp_time;
  o->unitTime = ctx->k.uTime;
  o->fluidHeight = ctx->fluidHeight;
  o->dem = ctx->demSolve;
  o->nObj = ctx->nObj;
  o->nWall = ctx->nWall;
  o->nBody = ctx->demSolve ? ctx->nBody : 0;
  o->slotDoubles = (size_t)o->nObj * OB_STRIDE + (size_t)o->nWall * 12 + STRESS_N +
                   (size_t)o->nBody * BD_STRIDE;
  o->vol = ctx->k.demSize[0] * ctx->k.demSize[1] * ctx->k.demSize[2];
  // realTime of the cycles already run, summed as goCycle sums it
  for (long long i = 0; i < ctx->lbTime; ++i) o->realTime += o->unitTime;
  const std::string d(dir);
  // IO::initialize, src/IO.cpp:8-94: its two data folders, then the files
  // (headers appended, as its ios::app opens)
  if (ctx->demSolve) ::mkdir((d + "/particleData").c_str(), 0777);
  if (ctx->lbSolve) ::mkdir((d + "/fluidData").c_str(), 0777);
  o->fExport = openWithHeader(d + "/export.dat", nullptr);
  bool ok = o->fExport != nullptr;
  if (o->dem) {
    o->fPos = openWithHeader(d + "/objPosition.dat",
                             "position(x) position(y) position(z) velocity(x) velocity(y) "
                             "velocity(z) depth(y)  \n");
    std::FILE* body = openWithHeader(d + "/bodyPosition.dat",
                                     "position(x) position(y) position(z) velocity(x) "
                                     "velocity(y) velocity(z) Length Delta  \n");
    o->fForce = openWithHeader(
        d + "/objForce.dat",
        "FExerted(x) FExerted(y) FExerted(z) SExerted(x) SExerted(y) SExerted(z) FTotal(x) "
        "FTotal(y) FTotal(z) FContact(x) FContact(y) FContact(z) FHydro(x) FHydro(y) "
        "FHydro(z) FLub(x) FLub(y) FLub(z) FRep(x) FRep(y) FRep(z) FGrav(x) FGrav(y) "
        "FGrav(z) \n");
    o->fWall = openWithHeader(
        d + "/wallForce.dat",
        "0-FTotal(x) 0-FTotal(y) 0-FTotal(z) 1-FTotal(x) 1-FTotal(y) 1-FTotal(z) 2-FTotal(x) "
        "2-FTotal(y) 2-FTotal(z) 3-FTotal(x) 3-FTotal(y) 3-FTotal(z) 4-FTotal(x) 4-FTotal(y) "
        "4-FTotal(z) 5-FTotal(x) 5-FTotal(y) 5-FTotal(z) \n");
    o->fStress = openWithHeader(d + "/stressTensor.dat", "xx yy zz xy yz zx \n");
    o->fNormal = openWithHeader(d + "/normalStressCont.dat",
                                "hydro-xx hydro-yy hydro-zz lub-xx lub-yy lub-zz contact-xx "
                                "contact-yy contact-zz rep-xx rep-yy rep-zz \n");
    o->fShear = openWithHeader(d + "/shearStressCont.dat",
                               "hydro-xy hydro-yz hydro-zx lub-xy lub-yz lub-zx contact-xy "
                               "contact-yz contact-zx rep-xy rep-yz rep-zx \n");
    ok = ok && o->fPos && body && o->fForce && o->fWall && o->fStress && o->fNormal && o->fShear;
    if (body && o->nBody > 0) o->fBody = body;
    else if (body) std::fclose(body);
  }
  if (!ok) {
    lbdemOutputFree(ctx);
    return fail(ctx, LBDEM_ERR_IO, std::string("output_open: cannot write files in ") + d);
  }
  o->slots.resize(kSlots);
  cudaError_t e = cudaMallocHost((void**)&o->pinned, kSlots * o->slotDoubles * sizeof(double));
  for (auto& s : o->slots)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    lbdemOutputFree(ctx);
    return fail(ctx, LBDEM_ERR_CUDA, std::string("output_open: ") + cudaGetErrorString(e));
  }
  // IO::outputStep before the first goCycle (src/main.cpp:286); a run that
  // has already cycled continues the schedule from its current time
  o->lastScreen = screenCounter(o, o->realTime);
  if (ctx->lbTime == 0 && o->lastScreen > 0) return capture(ctx);
  return LBDEM_OK;
}

extern "C" int lbdem_output_recycle(lbdem_ctx* ctx, double fluid_recycle_exp_time,
                                    double part_recycle_exp_time) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  lbdem_output* o = ctx->out;
  if (!o) return fail(ctx, LBDEM_ERR_INVALID, "output_recycle: output not open");
  if (!(fluid_recycle_exp_time >= 0.0) || !(part_recycle_exp_time >= 0.0))
    return fail(ctx, LBDEM_ERR_INVALID, "output_recycle: negative export time");
  o->recycleExp = ctx->lbSolve ? fluid_recycle_exp_time : 0.0;
  o->partExp = ctx->demSolve ? part_recycle_exp_time : 0.0;
  o->lastRecycle = recycleCounter(o, o->realTime);
  o->lastPart = partCounter(o, o->realTime);
  // the files IO::outputStep writes before the first goCycle
  if (ctx->lbTime != 0) return LBDEM_OK;
  if (o->lastRecycle > 0)
    if (int rc = writeRecycle(ctx)) return rc;
  if (o->lastPart > 0) return writePartRecycle(ctx, o->lastPart);
  return LBDEM_OK;
}

extern "C" int lbdem_output_close(lbdem_ctx* ctx) {
  if (!ctx) return LBDEM_ERR_INVALID;
  DeviceScope devScope(ctx->device);
  if (!ctx->out) return LBDEM_OK;
  const int rc = lbdemOutputDrain(ctx, true);
  lbdemOutputFree(ctx);
  return rc;
}
