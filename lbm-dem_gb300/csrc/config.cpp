// GetPot-format configuration and ./input/*.dat readers (host only).
//
// Replaces the parsing half of LB::latticeBoltzmannGet (src/LB.cpp:128-338),
// DEM::discreteElementGet (src/DEM.cpp:17-197) and parseConfigFile
// (src/main.cpp:128-185). The accepted syntax is the subset of GetPot the
// reference's inputs use: "key = value" tokens, '#' comments, double-quoted
// strings, and "-key value" command-line overrides that win over the file
// (src/macros.h:14-19). Value conversion follows GetPot's istream rules
// (getpot.h _convert_to_type): an integer key reads the leading integer of
// the token, a failed conversion yields the default.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "lbdem.h"

namespace {

struct KeyStore {
  std::map<std::string, std::string> file, cli;
  const std::string* find(const char* k) const {
    auto c = cli.find(k);
    if (c != cli.end()) return &c->second;
    auto f = file.find(k);
    if (f != file.end()) return &f->second;
    return nullptr;
  }
  double d(const char* k, double def) const {
    const std::string* s = find(k);
    if (!s) return def;
    std::istringstream in(*s);
    double v;
    in >> v;
    return in.fail() ? def : v;
  }
  int i(const char* k, int def) const {
    const std::string* s = find(k);
    if (!s) return def;
    std::istringstream in(*s);
    int v;
    in >> v;
    return in.fail() ? def : v;
  }
  bool b(const char* k, bool def) const {
    const std::string* s = find(k);
    if (!s) return def;
    std::string u(*s);
    for (char& c : u) c = (char)std::toupper((unsigned char)c);
    if (u.find("TRUE") != std::string::npos) return true;
    if (u.find("FALSE") != std::string::npos) return false;
    std::istringstream in(*s);
    unsigned v;
    in >> v;
    return in.fail() ? def : v != 0;
  }
  std::string s(const char* k, const char* def) const {
    const std::string* v = find(k);
    return v ? *v : std::string(def);
  }
};

// Tokenise a GetPot file into key -> value (last definition wins).
bool parseFile(const char* path, std::map<std::string, std::string>& out) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  std::vector<std::string> tok;
  while (std::getline(in, line)) {
    std::string cur;
    bool quoted = false;
    for (size_t k = 0; k < line.size(); ++k) {
      const char c = line[k];
      if (quoted) {
        if (c == '"') quoted = false;
        else cur += c;
        continue;
      }
      if (c == '#') break;
      if (c == '"') {
        quoted = true;
        continue;
      }
      if (c == '=') {
        if (!cur.empty()) tok.push_back(cur);
        cur.clear();
        tok.push_back("=");
        continue;
      }
      if (std::isspace((unsigned char)c)) {
        if (!cur.empty()) tok.push_back(cur);
        cur.clear();
        continue;
      }
      cur += c;
    }
    if (!cur.empty()) tok.push_back(cur);
  }
  for (size_t k = 0; k + 1 < tok.size(); ++k) {
    if (tok[k + 1] == "=" && tok[k] != "=") {
      std::string v = (k + 2 < tok.size() && tok[k + 2] != "=") ? tok[k + 2] : "";
      out[tok[k]] = v;
      k += v.empty() ? 1 : 2;
    }
  }
  return true;
}

void setErr(char* err, size_t n, const std::string& msg) {
  if (err && n) {
    std::snprintf(err, n, "%s", msg.c_str());
  }
}

}  // namespace

extern "C" int lbdem_config_defaults(lbdem_config* c) {
  if (!c) return LBDEM_ERR_INVALID;
  std::memset(c, 0, sizeof(*c));
  // src/main.cpp:128-185
  c->demInitialRepeat = 0.0;
  c->maxTime = 0.0;
  // src/LB.cpp:138-316
  c->unitLength = 1.0;
  c->unitTime = 1.0;
  c->unitDensity = 1.0;
  for (int k = 0; k < 3; ++k) c->lbRotCenter[k] = -1.0;
  for (int k = 0; k < 6; ++k) c->boundary[k] = 1;
  c->rheologyNewtonian = 1;
  c->initVisc = 1.0;
  // src/DEM.cpp:19-78
  c->scale = 1.0;
  return LBDEM_OK;
}

extern "C" int lbdem_config_load(const char* cfg_path, const char* input_dir,
                                 int argc, const char* const* argv,
                                 lbdem_config* c, char* err, size_t err_len) {
  if (!cfg_path || !c) return LBDEM_ERR_INVALID;
  lbdem_config_defaults(c);
  KeyStore ks;
  if (!parseFile(cfg_path, ks.file)) {
    setErr(err, err_len, std::string("cannot open config file ") + cfg_path);
    return LBDEM_ERR_IO;
  }
  for (int k = 0; k + 1 < argc; ++k) {
    const char* a = argv[k];
    if (a && a[0] == '-' && a[1] && !std::isdigit((unsigned char)a[1]) && a[1] != '.') {
      ks.cli[a + 1] = argv[k + 1] ? argv[k + 1] : "";
      ++k;
    }
  }
  c->demInitialRepeat = ks.d("demInitialRepeat", 0.0);
  c->lbmInitialRepeat = ks.i("lbmInitialRepeat", 0);
  c->maxTime = ks.d("maxTime", 0.0);
  c->maximumTimeSteps = ks.i("maximumTimeSteps", 0);
  c->screenExpTime = ks.d("screenExpTime", 0.0);
  c->fluidExpTime = ks.d("fluidExpTime", 0.0);
  c->fluidLagrangianExpTime = ks.d("fluidLagrangianExpTime", 0.0);
  c->partExpTime = ks.d("partExpTime", 0.0);
  c->fluidRecycleExpTime = ks.d("fluidRecycleExpTime", 0.0);
  c->partRecycleExpTime = ks.d("partRecycleExpTime", 0.0);
  c->demSolve = ks.i("demSolve", 0);
  c->lbSolve = ks.i("lbSolve", 0);
  c->freeSurfaceSolve = ks.i("freeSurfaceSolve", 0);
  c->forceFieldSolve = ks.i("forceFieldSolve", 0);

  c->lbRestart = ks.b("lbRestart", false);
  {
    const std::string f = ks.s("lbRestartFile", "");
    if (!f.empty()) {
      char* p = new char[f.size() + 1];
      std::memcpy(p, f.c_str(), f.size() + 1);
      c->lbRestartFile = p;
    }
  }
  c->lbTopography = ks.b("lbTopography", false);
  c->unitLength = ks.d("unitLength", 1.0);
  c->unitTime = ks.d("unitTime", 1.0);
  c->unitDensity = ks.d("unitDensity", 1.0);
  c->lbSizeX = ks.d("lbSizeX", 0.0);
  c->lbSizeY = ks.d("lbSizeY", 0.0);
  c->lbSizeZ = ks.d("lbSizeZ", 0.0);
  // src/LB.cpp:196-242: each model reads its own keys; the others keep
  // FluidMaterial's defaults (src/node.h:41-50), initVisc 1/6 included
  const std::string rheo = ks.s("rheologyModel", "none");
  c->rheologyModel = rheo == "BINGHAM" ? LBDEM_BINGHAM
                   : rheo == "FRICTIONAL" ? LBDEM_FRICTIONAL
                   : rheo == "VOELLMY" ? LBDEM_VOELLMY : LBDEM_NEWTONIAN;
  c->rheologyNewtonian = c->rheologyModel == LBDEM_NEWTONIAN ? 1 : 0;
  c->initVisc = (1.0 - 0.5) / 3.0;
  c->voellmyConstant = 0.0;
  if (c->rheologyModel != LBDEM_BINGHAM) c->initVisc = ks.d("initVisc", 1.0);
  if (c->rheologyModel == LBDEM_BINGHAM) {
    c->plasticVisc = ks.d("plasticVisc", 0.0);
    c->yieldStress = ks.d("yieldStress", 0.0);
  }
  if (c->rheologyModel == LBDEM_FRICTIONAL || c->rheologyModel == LBDEM_VOELLMY)
    c->frictionCoefFluid = ks.d("frictionCoefFluid", 0.0);
  if (c->rheologyModel == LBDEM_VOELLMY) c->voellmyConstant = ks.d("voellmyConstant", 1.0);
  c->turbulenceSolve = ks.i("turbulenceSolve", 0);
  c->turbConst = ks.d("turbConst", 0.0);
  c->initVelocity[0] = ks.d("initVelocityX", 0.0);
  c->initVelocity[1] = ks.d("initVelocityY", 0.0);
  c->initVelocity[2] = ks.d("initVelocityZ", 0.0);
  c->lbF[0] = ks.d("lbFX", 0.0);
  c->lbF[1] = ks.d("lbFY", 0.0);
  c->lbF[2] = ks.d("lbFZ", 0.0);
  c->lbRot[0] = ks.d("lbRotX", 0.0);
  c->lbRot[1] = ks.d("lbRotY", 0.0);
  c->lbRot[2] = ks.d("lbRotZ", 0.0);
  c->lbRotCenter[0] = ks.d("lbRotCenterX", -1.0);
  c->lbRotCenter[1] = ks.d("lbRotCenterY", -1.0);
  c->lbRotCenter[2] = ks.d("lbRotCenterZ", -1.0);
  const char* bnames[6] = {"boundary0", "boundary1", "boundary2",
                           "boundary3", "boundary4", "boundary5"};
  for (int k = 0; k < 6; ++k) c->boundary[k] = ks.i(bnames[k], 1);
  c->slipCoefficient = ks.d("slipCoefficient", 0.0);
  c->fluidHeight = ks.d("fluidHeight", 0.0);

  c->density = ks.d("density", 0.0);
  c->objectDensity = ks.d("objectDensity", 0.0);
  c->bodyDensity = ks.d("bodyDensity", 0.0);
  c->linearStiff = ks.d("linearStiff", 0.0);
  c->frictionCoefPart = ks.d("frictionCoefPart", 0.0);
  c->lubNormal = ks.d("lubNormal", 0.0);
  c->lubTangential = ks.d("lubTangential", 0.0);
  c->lubRotation = ks.d("lubRotation", 0.0);
  c->lubCutoff = ks.d("lubCutoff", 0.0);
  c->kinVisc = ks.d("kinVisc", 0.0);
  c->electroForce = ks.d("electroForce", 0.0);
  c->debyeLength = ks.d("debyeLength", 0.0);
  c->objWaitTime = ks.i("objWaitTime", 0);
  c->intervalTime = ks.i("intervalTime", 0);
  c->springDamp = ks.d("springDamp", 0.0);
  c->epsilon = ks.d("epsilon", 0.0);
  c->nonLinType = ks.i("nonLinType", 0);
  c->k13 = ks.d("k13", 0.0);
  c->scale = ks.d("scale", 1.0);

  // ./input/particles.dat, src/DEM.cpp:80-134
  const std::string dir = input_dir ? input_dir : "./input";
  const double scale = c->scale;
  {
    std::ifstream in(dir + "/particles.dat");
    if (!in) {
      setErr(err, err_len, "cannot open " + dir + "/particles.dat");
      return LBDEM_ERR_IO;
    }
    unsigned tot = 0;
    in >> tot;
    auto* ps = new lbdem_particle_in[tot ? tot : 1]();
    for (unsigned n = 0; n < tot; ++n) {
      lbdem_particle_in& p = ps[n];
      unsigned idx = 0, size = 1;
      double q[8];
      in >> idx >> size >> p.r;
      p.r = p.r * scale;
      double x0, y0, z0;
      in >> x0 >> y0 >> z0;
      p.x[0] = x0 * scale - 0.05;
      p.x[1] = y0 * scale - 0.05;
      p.x[2] = z0 * scale - 0.05;
      in >> p.v[0] >> p.v[1] >> p.v[2] >> p.w[0] >> p.w[1] >> p.w[2];
      for (double& v : q) in >> v;
      p.size = (int32_t)size;
      p.index = (int32_t)idx;
      if (!in) {
        delete[] ps;
        setErr(err, err_len, "malformed particles.dat");
        return LBDEM_ERR_IO;
      }
    }
    c->n_particles = (int32_t)tot;
    c->particles = ps;
  }
  // ./input/objects.dat, src/DEM.cpp:137-166
  {
    std::ifstream in(dir + "/objects.dat");
    if (!in) {
      lbdem_config_release(c);
      setErr(err, err_len, "cannot open " + dir + "/objects.dat");
      return LBDEM_ERR_IO;
    }
    unsigned tot = 0;
    in >> tot;
    auto* os = new lbdem_object_in[tot ? tot : 1]();
    for (unsigned n = 0; n < tot; ++n) {
      lbdem_object_in& o = os[n];
      unsigned idx = 0;
      in >> idx >> o.r;
      o.index = (int32_t)idx;
      o.r = o.r * scale;
      double x0, y0, z0;
      in >> x0 >> y0 >> z0;
      o.x[0] = x0 * scale;
      o.x[1] = y0 * scale;
      o.x[2] = z0 * scale;
      in >> o.v[0] >> o.v[1] >> o.v[2];
      if (!in) {
        delete[] os;
        lbdem_config_release(c);
        setErr(err, err_len, "malformed objects.dat");
        return LBDEM_ERR_IO;
      }
    }
    c->n_objects = (int32_t)tot;
    c->objects = os;
  }
  // ./input/body.dat, src/DEM.cpp:168-196 (only an empty list is supported)
  {
    std::ifstream in(dir + "/body.dat");
    if (!in) {
      lbdem_config_release(c);
      setErr(err, err_len, "cannot open " + dir + "/body.dat");
      return LBDEM_ERR_IO;
    }
    unsigned tot = 0;
    in >> tot;
    auto* bs = new lbdem_body_in[tot ? tot : 1]();
    for (unsigned n = 0; n < tot; ++n) {
      lbdem_body_in& b = bs[n];
      unsigned idx = 0;
      double x0, y0, z0;
      in >> idx >> b.r >> x0 >> y0 >> z0 >> b.v[0] >> b.v[1] >> b.v[2] >> b.k >> b.L0;
      b.index = (int32_t)idx;
      b.x[0] = x0 * scale;
      b.x[1] = y0 * scale;
      b.x[2] = z0 * scale;
      if (!in) {
        delete[] bs;
        lbdem_config_release(c);
        setErr(err, err_len, "malformed body.dat");
        return LBDEM_ERR_IO;
      }
    }
    c->n_bodies = (int32_t)tot;
    c->bodies = bs;
  }
  return LBDEM_OK;
}

extern "C" void lbdem_config_release(lbdem_config* c) {
  if (!c) return;
  delete[] c->particles;
  delete[] c->objects;
  delete[] c->lbRestartFile;
  delete[] c->bodies;
  c->bodies = nullptr;
  c->n_bodies = 0;
  c->particles = nullptr;
  c->objects = nullptr;
  c->lbRestartFile = nullptr;
  c->n_particles = c->n_objects = 0;
}
