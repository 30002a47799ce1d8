// lbdem_run: command-line driver of an impact run through the C ABI, in the
// place of the reference's main (src/main.cpp:200-310).
//
//   lbdem_run [-c config.cfg] [-i inputDir] [-d dataDir] [-n name]
//             [-precision fp64|mixed] [-device k] [-steps n] [-every n]
//             [-resume snapshot] [-snapshot snapshot] [-key value ...]
//
// As in the reference: the GetPot parameters file is read from -c (default
// config.cfg); the particles/objects/body tables from input/ relative to the
// working directory (-i changes that); the config file is copied into the
// data directory (-d, default "data", plus /name with -n); any "-key value"
// pair overrides the key of the parameters file; and the run goes on until
// the simulated time passes maxTime (goCycle adds unitTime per cycle,
// src/main.cpp:38-67, 290-305). Additions:
// - -steps n stops after n cycles (maxTime = 0 with no -steps runs 0 cycles);
// - -precision chooses the plain FP64 form (default, reference-exact) or the
//   mixed form;
// - every -every cycles (default: every screenExpTime of simulated time, or
//   only at the end) one line per impactor goes to <data>/impactor.dat and a
//   summary line to stdout;
// - -resume loads a snapshot (lbdem_restore) of a run of the same
//   parameters and form before the first cycle; the run goes on from the
//   snapshot's cycle count, -steps and maxTime still counting from cycle 0,
//   and impactor.dat is appended to;
// - -snapshot writes a snapshot (lbdem_checkpoint) after the last cycle.
//   Both replace the reference's recycle/restart files (src/IO.cpp:973-997,
//   src/LB.cpp:353-367) with a bit-exact state.
// With screenExpTime > 0 the reference's own screen-phase files (export.dat,
// objPosition.dat, objForce.dat, wallForce.dat, ...) are written into the
// data directory as IO::outputStep writes them (lbdem_output_open), and with
// fluidRecycleExpTime / partRecycleExpTime > 0 its recycle files into
// data/fluidData and data/particleData (lbdem_output_recycle).
#include <sys/stat.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "lbdem.h"

namespace {

const char* flagValue(int argc, char** argv, const char* flag, const char* def) {
  for (int k = 1; k + 1 < argc; ++k)
    if (std::strcmp(argv[k], flag) == 0) return argv[k + 1];
  return def;
}
bool hasFlag(int argc, char** argv, const char* flag) {
  for (int k = 1; k < argc; ++k)
    if (std::strcmp(argv[k], flag) == 0) return true;
  return false;
}

bool makeDir(const std::string& d) {
  return ::mkdir(d.c_str(), 0777) == 0 || errno == EEXIST;
}

int fail(lbdem_ctx* ctx, const char* what, int rc) {
  std::fprintf(stderr, "lbdem_run: %s failed (status %d): %s\n", what, rc,
               ctx ? lbdem_last_error(ctx) : "");
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (hasFlag(argc, argv, "-h") || hasFlag(argc, argv, "--help")) {
    std::printf(
        "Usage: %s [-c configFile] [-i inputDir] [-d dataDir] [-n name] "
        "[-precision fp64|mixed] [-device k] [-steps n] [-every n] [-resume snapshot] "
        "[-snapshot snapshot] [-key value ...]\n",
        argv[0]);
    return 0;
  }
  const std::string cfgPath = flagValue(argc, argv, "-c", "config.cfg");
  const std::string inputDir = flagValue(argc, argv, "-i", "input");
  std::string workDir = flagValue(argc, argv, "-d", "data");
  const std::string name = flagValue(argc, argv, "-n", "");
  const std::string precision = flagValue(argc, argv, "-precision", "fp64");
  const int device = std::atoi(flagValue(argc, argv, "-device", "0"));
  const long long stepLimit = std::atoll(flagValue(argc, argv, "-steps", "-1"));
  const long long every = std::atoll(flagValue(argc, argv, "-every", "0"));
  const std::string resume = flagValue(argc, argv, "-resume", "");
  const std::string snapshot = flagValue(argc, argv, "-snapshot", "");
  if (precision != "fp64" && precision != "mixed") {
    std::fprintf(stderr, "lbdem_run: -precision must be fp64 or mixed\n");
    return 1;
  }

  lbdem_config cfg;
  char err[1024];
  int rc = lbdem_config_load(cfgPath.c_str(), inputDir.c_str(), argc - 1,
                             (const char* const*)(argv + 1), &cfg, err, sizeof err);
  if (rc) {
    std::fprintf(stderr, "lbdem_run: reading %s: %s\n", cfgPath.c_str(), err);
    return 1;
  }
  if (!makeDir(workDir)) {
    std::fprintf(stderr, "lbdem_run: cannot create %s\n", workDir.c_str());
    return 1;
  }
  if (!name.empty()) {
    workDir += "/" + name;
    if (!makeDir(workDir)) {
      std::fprintf(stderr, "lbdem_run: cannot create %s\n", workDir.c_str());
      return 1;
    }
  }
  {  // keep the parameters with the results, as the reference does
    std::ifstream src(cfgPath, std::ios::binary);
    std::ofstream dst(workDir + "/" + cfgPath.substr(cfgPath.find_last_of('/') + 1),
                      std::ios::binary);
    dst << src.rdbuf();
  }

  lbdem_options opt;
  std::memset(&opt, 0, sizeof opt);
  opt.precision = precision == "mixed" ? LBDEM_MIXED : LBDEM_PLAIN_FP64;
  opt.device = device;
  lbdem_ctx* ctx = nullptr;
  if ((rc = lbdem_create(&cfg, &opt, &ctx))) {
    const int code = fail(ctx, "lbdem_create", rc);
    lbdem_destroy(ctx);
    lbdem_config_release(&cfg);
    return code;
  }
  lbdem_info info;
  if ((rc = lbdem_get_info(ctx, &info))) return fail(ctx, "lbdem_get_info", rc);
  const int nObj = info.n_objects;
  std::printf("lbdem_run: %dx%dx%d lattice, %d particles, %d impactor(s), %s form, %.3f GB\n",
              info.lb_size[0], info.lb_size[1], info.lb_size[2], info.n_particles, nObj,
              precision.c_str(), info.device_bytes / 1e9);

  // number of goCycles: the reference's loop adds unitTime to realTime per
  // cycle until realTime > maxTime
  long long total = 0;
  {
    double realTime = 0.0;
    while (!(realTime != 0.0 && realTime > cfg.maxTime)) {
      if (stepLimit >= 0 && total >= stepLimit) break;
      realTime += cfg.unitTime;
      ++total;
      if (stepLimit < 0 && total > (1LL << 40)) break;  // maxTime out of reach
    }
  }
  long long interval = every;
  if (interval <= 0 && cfg.screenExpTime > 0.0)
    interval = (long long)(cfg.screenExpTime / cfg.unitTime + 0.5);
  if (interval <= 0) interval = total > 0 ? total : 1;

  long long done = 0;
  if (!resume.empty()) {
    if ((rc = lbdem_restore(ctx, resume.c_str()))) return fail(ctx, "lbdem_restore", rc);
    if ((rc = lbdem_get_info(ctx, &info))) return fail(ctx, "lbdem_get_info", rc);
    done = info.time_step;
    std::printf("lbdem_run: resumed at cycle %lld from %s\n", done, resume.c_str());
  }
  std::FILE* out =
      std::fopen((workDir + "/impactor.dat").c_str(), resume.empty() ? "w" : "a");
  if (!out) {
    std::fprintf(stderr, "lbdem_run: cannot write %s/impactor.dat\n", workDir.c_str());
    return 1;
  }
  if (resume.empty()) std::fprintf(out, "# step time object x y z vx vy vz FHx FHy FHz\n");
  std::vector<double> x0(3 * (nObj > 0 ? nObj : 1)), x1(x0.size()), fh(x0.size());
  auto report = [&](long long step) -> int {
    lbdem_object_view v;
    std::memset(&v, 0, sizeof v);
    v.x0 = x0.data();
    v.x1 = x1.data();
    v.FHydro = fh.data();
    int r = lbdem_download_objects(ctx, &v);
    if (r) return r;
    double mass = 0.0;
    int64_t nIf = 0, nAct = 0;
    if ((r = lbdem_mass_summary(ctx, &mass, &nIf, &nAct))) return r;
    const double t = step * cfg.unitTime;
    for (int o = 0; o < nObj; ++o)
      std::fprintf(out, "%lld %.17g %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n",
                   step, t, o, x0[3 * o], x0[3 * o + 1], x0[3 * o + 2], x1[3 * o],
                   x1[3 * o + 1], x1[3 * o + 2], fh[3 * o], fh[3 * o + 1], fh[3 * o + 2]);
    std::printf("step %lld time %.6g fluid mass %.12g interface %lld active %lld", step, t, mass,
                (long long)nIf, (long long)nAct);
    if (nObj > 0) std::printf(" impactor y %.9g", x0[1]);
    std::printf("\n");
    return 0;
  };

  if (cfg.screenExpTime > 0.0 || cfg.fluidRecycleExpTime > 0.0 ||
      cfg.partRecycleExpTime > 0.0) {
    if ((rc = lbdem_output_open(ctx, workDir.c_str(), cfg.screenExpTime)))
      return fail(ctx, "lbdem_output_open", rc);
    if ((rc = lbdem_output_recycle(ctx, cfg.fluidRecycleExpTime, cfg.partRecycleExpTime)))
      return fail(ctx, "lbdem_output_recycle", rc);
  }
  if (resume.empty() && (rc = report(0))) return fail(ctx, "report", rc);
  while (done < total) {
    const long long n = total - done < interval ? total - done : interval;
    if ((rc = lbdem_cycle(ctx, (int32_t)n))) return fail(ctx, "lbdem_cycle", rc);
    done += n;
    if ((rc = lbdem_sync(ctx))) return fail(ctx, "lbdem_sync", rc);
    if ((rc = report(done))) return fail(ctx, "report", rc);
  }
  std::fclose(out);
  if ((rc = lbdem_output_close(ctx))) return fail(ctx, "lbdem_output_close", rc);
  if (!snapshot.empty()) {
    if ((rc = lbdem_checkpoint(ctx, snapshot.c_str()))) return fail(ctx, "lbdem_checkpoint", rc);
    std::printf("lbdem_run: snapshot of cycle %lld in %s\n", done, snapshot.c_str());
  }
  lbdem_destroy(ctx);
  lbdem_config_release(&cfg);
  std::printf("lbdem_run: %lld cycles done, results in %s\n", done, workDir.c_str());
  return 0;
}
