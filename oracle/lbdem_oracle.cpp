// CPU restatement of the reference's coupled free-surface LB / DEM step.
//
// TEST INFRASTRUCTURE ONLY (see lbdem_oracle.h). Serial, dense-array
// restatement of the reference algorithm in the reference's own floating
// point operation order, so that it agrees with the pinned reference build
// bit for bit. Every function cites the reference lines it restates
// (paths relative to the reference project root).
//
// Reference quirks that are reproduced on purpose:
//  * LB::findNewActive (src/LB.cpp:1985-2017): the `break` leaves the loop
//    over particleNodes at the first node still inside its particle, so only
//    the leading run of uncovered nodes is un-flagged.
//  * LB::findNewSolid (src/LB.cpp:2045-2098): the `break` leaves the k loop
//    before the append block, so no node is ever flagged here.
//  * LB::initializeParticleBoundaries (src/LB.cpp:689-693) resets the solid
//    index of every node, walls included, to 0.
//  * LB::findNewActiveObject uses object 0 for every object node
//    (src/LB.cpp:870).
//  * DEM::initializeWalls takes slip/moving flags from boundary[0] only
//    (src/DEM.cpp:430-448).
//  * object-particle tangential damping dampCoeffTanw is an uninitialised
//    local (src/DEM.cpp:916), zero under the defined-behaviour pin.
// Not reproduced: the reference stores solid indices in 16 bits
// (src/node.h:148); this restatement keeps 32 bits (identical below 65536
// particles).
#include "lbdem_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <omp.h>

#include "statedump.h"

namespace {

// ---- lattice constants, src/lattice.h:33-150 ----------------------------
const double V[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},
                         {0, -1, 0}, {0, 0, 1},  {0, 0, -1}, {1, 1, 0},
                         {-1, -1, 0}, {-1, 1, 0}, {1, -1, 0}, {0, 1, 1},
                         {0, -1, -1}, {0, -1, 1}, {0, 1, -1}, {1, 0, 1},
                         {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1}};
const unsigned OPP[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
const unsigned SLIP1C[19] = {0, 0, 0, 0, 0, 0, 0, 1, 2, 3, 4, 3, 4, 5, 6, 1, 2, 6, 5};
const unsigned SLIP1[19] = {0, 0, 0, 0, 0, 0, 0, 9, 10, 8, 7, 13, 14, 12, 11, 18, 17, 15, 16};
const unsigned SLIP2C[19] = {0, 0, 0, 0, 0, 0, 0, 3, 4, 2, 1, 5, 6, 4, 3, 5, 6, 1, 2};
const unsigned SLIP2[19] = {0, 0, 0, 0, 0, 0, 0, 10, 9, 7, 8, 14, 13, 11, 12, 17, 18, 16, 15};
const double COEFF[19] = {12.0 / 36.0, 2.0 / 36.0, 2.0 / 36.0, 2.0 / 36.0, 2.0 / 36.0,
                          2.0 / 36.0,  2.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                          1.0 / 36.0,  1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                          1.0 / 36.0,  1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
const double PI = 3.14159265358979323846;  // M_PI, src/myvector.h:6

// ---- 3-vector with the reference's component-wise semantics -------------
// (src/myvector.cpp:48-146)
struct Vec {
  double x = 0.0, y = 0.0, z = 0.0;
  Vec() = default;
  Vec(double a, double b, double c) : x(a), y(b), z(c) {}
};
inline Vec operator+(Vec a, Vec b) { return Vec(a.x + b.x, a.y + b.y, a.z + b.z); }
inline Vec operator-(Vec a, Vec b) { return Vec(a.x - b.x, a.y - b.y, a.z - b.z); }
inline Vec operator*(Vec a, double s) { return Vec(a.x * s, a.y * s, a.z * s); }
inline Vec operator*(double s, Vec a) { return Vec(a.x * s, a.y * s, a.z * s); }
inline Vec operator/(Vec a, double s) { return Vec(a.x / s, a.y / s, a.z / s); }
inline Vec& operator+=(Vec& a, Vec b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  return a;
}
inline Vec& operator*=(Vec& a, double s) {
  a.x *= s;
  a.y *= s;
  a.z *= s;
  return a;
}
inline double dot(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double norm2(Vec a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline Vec cross(Vec a, Vec b) {
  return Vec(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline Vec vdir(int j) { return Vec(V[j][0], V[j][1], V[j][2]); }
// tinyVector::insideSphere, src/myvector.cpp:171-176
inline bool insideSphere(Vec p, Vec c, double r) { return norm2(p - c) < r * r; }
// tinyVector::insidePlane, src/myvector.cpp:222-225
inline bool insidePlane(Vec p, Vec w, Vec n) { return dot(n, p - w) < 0.0; }

// DEM.cpp helper macros, src/DEM.cpp:5-12
inline int n_int(double x) { return x >= 0 ? (int)(x + 0.5) : (int)(x - 0.5); }
inline int s_int(double x) { return x >= 0 ? (int)(x) : (int)(x - 1.0); }
inline double box(double a, double b) { return a - s_int(a / b) * b; }
inline double n_image(double a, double b) { return a - n_int(a / b) * b; }
inline double dmax(double a, double b) { return a > b ? a : b; }

// ---- DEM element types, src/elmt.h:15-228, src/utils.h:19-101 -----------
const int MAX_N = 50;  // src/DEM.cpp:476
struct Particle {
  double r = 1.0, m = 1.0, I = 1.0, _m = 1.0, _I = 1.0, dens = 1.0;
  unsigned size = 1, particleIndex = 0;
  Vec x0, x1, w1;
  Vec FHydro, FContact, FTotal, FLub, FGrav, FRep;
  Vec MHydro, MContact, MTotal, MLub;
  Vec xiw, xio;
  double fluidVolume = 0.0;
  double SHydro[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int list[MAX_N] = {0}, _list[MAX_N] = {0};
  double xix[MAX_N] = {0}, xiy[MAX_N] = {0}, xiz[MAX_N] = {0};
  double _xix[MAX_N] = {0}, _xiy[MAX_N] = {0}, _xiz[MAX_N] = {0};
};
struct Object {
  unsigned index = 0;
  double r = 0.0, m = 1.0, _m = 1.0, I = 1.0, _I = 1.0;
  Vec x0, x1, w1;
  Vec FContact, FHydro, FLub, FGrav, FSpring, FTotal;
  Vec MContact, MHydro, MTotal, MLub;
};
// body, src/elmt.h:231-258
struct Body {
  unsigned index = 0;
  double r = 1.0, m = 1.0, _m = 1.0, L0 = 1.0, L = 1.0, k = 1.0;
  Vec x0, x1;
  Vec FGrav, FSpring, FTotal;
};
struct Wall {
  unsigned index = 0;
  Vec n{1, 0, 0}, p;
  bool moving = false, slip = false;
  Vec FHydro, FContact, FLub, FTotal, FRep;
};

}  // namespace

struct oracle_ctx {
  std::string err;
  // run switches, src/main.cpp:128-185
  bool demSolve = false, lbSolve = false;
  // ---- LB (src/LB.h:32-230) ----
  bool freeSurface = false, forceField = false;
  double uLength = 1, uTime = 1, uDensity = 1, uVolume = 1, uSpeed = 1, uAccel = 1,
         uAngVel = 1, uForce = 1, uTorque = 1, uKinVisc = 1, uDynVisc = 1;
  int X = 1, Y = 1, Z = 1;
  size_t N = 0;
  long ne[19] = {0};
  double physSize[3] = {0, 0, 0};
  Vec boundaryLoc[6];
  int boundary[6] = {1, 1, 1, 1, 1, 1};
  double slipCoefficient = 0.0, fluidHeight = 0.0;
  double initDensity = 1.0, initDynVisc = 0.0;
  // FluidMaterial's rheology (src/node.h:19-50), in lattice units
  int rheology = LBDEM_NEWTONIAN;
  double plasticVisc = 0.0, yieldStress = 0.0, frictionCoefFluid = 0.0, voellmyCoefficient = 0.0;
  bool turbulenceOn = false;
  double turbConst = 0.0;
  Vec initVelocity, lbF;
  unsigned lbTime = 0;
  std::vector<uint8_t> t, p, hasnode;
  std::vector<uint32_t> solid;
  std::vector<double> f, fs, n, ux, uy, uz, hx, hy, hz, mass, newMass, visc;
  std::vector<unsigned> fluidNodes, interfaceNodes, particleNodes, activeNodes, objectNodes;
  // ---- DEM (src/DEM.h:21-190) ----
  double demSize[3] = {1, 1, 1}, vol = 1, deltat = 1.0, demTime = 0.0,
         demInitialRepeat = 0.0;
  unsigned demTimeStep = 0;
  int objWaitTime = 0;
  double density = 1, objectDensity = 1, linearStiff = 0, dampCoeff = 0,
         frictionCoefPart = 0, lubNormal = 0, lubTangential = 0, lubRotation = 0,
         lubCutoff = 0, kinVisc = 0, electroForce = 0, debyeLength = 0;
  Vec demF;
  std::vector<Body> bodies;
  double bodyDensity = 0.0, springDamp = 0.0, k13 = 0.0, epsilon = 0.0;
  int nonLinType = 0;
  double maxDisp = 0.0, minPartRadius = 0, maxPartRadius = 0, meanPartRadius = 0;
  bool newNeighborList = false;
  std::vector<Particle> particles;
  std::vector<Object> objects;
  std::vector<Wall> walls;
  int64_t rebuilds = 0;
  std::vector<int> cellList;  // [MAX_L][MAX_N+1], src/DEM.cpp:479-481

  // ------------------------------------------------------------------------
  // index helpers, src/LB.cpp:2113-2169
  unsigned getX(size_t i) const { return (unsigned)((i % ((size_t)X * Y)) % X); }
  unsigned getY(size_t i) const { return (unsigned)((i % ((size_t)X * Y)) / X); }
  unsigned getZ(size_t i) const { return (unsigned)(i / ((size_t)X * Y)); }
  Vec pos(size_t i) const { return Vec(double(getX(i)), double(getY(i)), double(getZ(i))); }
  bool isActive(size_t i) const { return t[i] == 0 || t[i] == 3; }
  bool isWall(size_t i) const { return t[i] >= 5 && t[i] <= 11; }
  double& F(int j, size_t i) { return f[(size_t)j * N + i]; }
  double& FS(int j, size_t i) { return fs[(size_t)j * N + i]; }
  Vec U(size_t i) const { return Vec(ux[i], uy[i], uz[i]); }
  void setU(size_t i, Vec v) {
    ux[i] = v.x;
    uy[i] = v.y;
    uz[i] = v.z;
  }
  Vec H(size_t i) const { return Vec(hx[i], hy[i], hz[i]); }
  // neighbour table of a node, src/LB.cpp:567-618 (no periodic nodes here)
  long link(size_t it, int j) const {
    long d = (long)it + ne[j];
    if (isWall(it)) {
      const unsigned x = getX(it), y = getY(it), z = getZ(it);
      if ((x == 0 && V[j][0] < 0.0) || (x == (unsigned)X - 1 && V[j][0] > 0.0) ||
          (y == 0 && V[j][1] < 0.0) || (y == (unsigned)Y - 1 && V[j][1] > 0.0) ||
          (z == 0 && V[j][2] < 0.0) || (z == (unsigned)Z - 1 && V[j][2] > 0.0))
        d = (long)it;
    }
    return d;
  }

  // ---- node operations, src/node.cpp -------------------------------------
  // node::node() via LB::createNode, src/node.h:79-94, src/LB.cpp:476-483
  void createNode(size_t i) {
    hasnode[i] = 1;
    n[i] = 0.0;
    ux[i] = uy[i] = uz[i] = 0.0;
    hx[i] = hy[i] = hz[i] = 0.0;
    mass[i] = newMass[i] = 0.0;
    for (int j = 0; j < 19; ++j) F(j, i) = FS(j, i) = 0.0;
  }
  // node::setEquilibrium, src/node.cpp:52-73
  void setEquilibrium(size_t i) {
    const Vec u = U(i);
    const double usq = norm2(u);
    for (int j = 0; j < 19; ++j) {
      const double vu = dot(u, vdir(j));
      F(j, i) = FS(j, i) = COEFF[j] * n[i] * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
    }
  }
  // node::initialize, src/node.cpp:26-36
  void initialize(size_t i, double density, Vec velocity, double massFunction,
                  double viscosity, Vec force) {
    n[i] = density;
    mass[i] = massFunction;
    setU(i, force / 2.0 / n[i] + velocity);
    visc[i] = viscosity;
    setEquilibrium(i);
  }
  // node::reconstruct, src/node.cpp:75-93
  void reconstruct(size_t i) {
    double nn = 0.0;
    for (int j = 0; j < 19; ++j) nn += F(j, i);
    Vec u;
    for (int j = 0; j < 19; ++j) u += F(j, i) * vdir(j);
    n[i] = nn;
    setU(i, u / nn);
  }
  // node::computeEquilibrium, src/node.cpp:100-111
  void computeEquilibrium(size_t i, double* feq) const {
    const Vec u = U(i);
    const double usq = norm2(u);
    for (int j = 0; j < 19; ++j) {
      const double vu = dot(u, vdir(j));
      feq[j] = COEFF[j] * n[i] * (1.0 + 3.0 * vu + 4.5 * vu * vu - 1.5 * usq);
    }
  }
  // node::computeApparentViscosity, src/node.cpp:113-168: the shear-rate
  // tensor from the non-equilibrium populations, with the node's viscosity
  // of the last step in tau; the model's apparent viscosity (plus the
  // Smagorinsky term) clamped to the viscosities of tau 0.500001 and 1.8
  // (src/lattice.h:26-27). Terms with c_a c_b = 0 add nothing (and leave
  // every sum's bits as they are), c_a c_b = +-1 adds or subtracts.
  void computeApparentViscosity(size_t i, const double* feq) {
    const double minVisc = (0.500001 - 0.5) / 3.0;
    const double maxVisc = (1.8 - 0.5) / 3.0;
    const double tau = 0.5 + 3.0 * visc[i];
    double g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < 19; ++j) {
      const double d = F(j, i) - feq[j];
      const int c[3] = {(int)V[j][0], (int)V[j][1], (int)V[j][2]};
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          const int cc = c[a] * c[b];
          if (cc > 0) g[3 * a + b] += d;
          else if (cc < 0) g[3 * a + b] += -d;
        }
    }
    const double sc = 1.5 / (tau * n[i]);
    for (double& v : g) v *= sc;
    const double mag = std::sqrt(0.5 * (g[0] * g[0] + g[4] * g[4] + g[8] * g[8] +
                                        2.0 * (g[1] * g[3] + g[6] * g[2] + g[5] * g[7])));
    const double shearRate = 2.0 * mag;
    double nuApp = 0.0;
    const Vec u = U(i);
    if (rheology == LBDEM_BINGHAM) {
      nuApp = plasticVisc + yieldStress / shearRate;
    } else if (rheology == LBDEM_FRICTIONAL) {
      const double pressure = std::max(0.0, 0.33333333 * (n[i] - 1.0));
      nuApp = initDynVisc + frictionCoefFluid * pressure / shearRate;
    } else if (rheology == LBDEM_VOELLMY) {
      const double pressure = std::max(0.0, 0.33333333 * (n[i] - 1.0));
      nuApp = (frictionCoefFluid * pressure + norm2(u) / voellmyCoefficient) / shearRate;
    } else {
      nuApp = initDynVisc;
    }
    if (turbulenceOn) {
      const double nuTurb = turbConst * shearRate;
      nuApp += nuTurb;
    }
    visc[i] = std::max(minVisc, std::min(maxVisc, nuApp));
  }
  // node::bounceBackForce, src/node.cpp:306-314
  Vec bounceBackForce(size_t i, int j, const double* sp, double BBi) {
    return (2.0 * (FS(j, i) - sp[j]) - BBi) * vdir(j);
  }
  // node::massStream, src/node.cpp:316-318
  double massStream(size_t i, int j) { return F(OPP[j], i) - FS(j, i); }

  // ------------------------------------------------------------------------
  int init(const lbdem_config* c);
  void lbInit();
  void demInit();
  void initializeLists();
  void cleanLists();
  void updateObjectBoundaries();
  void updateIndices();
  void findNewActive();
  void computeHydroForces();
  void collision();
  void streaming();
  void redistributeMass(double s);
  void updateMass();
  void updateInterface();
  void couplingStep();
  void lbStep();
  void fsStep();
  void demStep();
  void neighborList();
  void evaluateForces();
  void integration();
  void bodyObjectInteraction();
  void particleContact();
  void particleLubrication();
  void particleElectro();
  void wallContact(bool fictional);
  void wallLubrication();
  void objectContact();
  void objectLubrication();
  void goCycle();
  void dump(const char* path);
};

// ==== initialisation =======================================================

int oracle_ctx::init(const lbdem_config* c) {
  if (c->lbRestart || c->lbTopography) {
    err = "restart and topography are not supported";
    return LBDEM_ERR_INVALID;
  }
  bodies.resize(c->n_bodies);
  for (int b = 0; b < c->n_bodies; ++b) {  // DEM::discreteElementGet, src/DEM.cpp:168-196
    const lbdem_body_in& in = c->bodies[b];
    Body& d = bodies[b];
    d.index = (unsigned)in.index;
    d.r = in.r;
    d.x0 = Vec(in.x[0], in.x[1], in.x[2]);
    d.x1 = Vec(in.v[0], in.v[1], in.v[2]);
    d.k = in.k;
    d.L0 = in.L0;
  }
  bodyDensity = c->bodyDensity;
  springDamp = c->springDamp;
  nonLinType = c->nonLinType;
  k13 = c->k13;
  epsilon = c->epsilon;
  for (int k = 0; k < 6; ++k)
    if (c->boundary[k] == 4 || c->boundary[k] == 9 || c->boundary[k] == 1) {
      err = "periodic/cylinder boundaries are not supported";
      return LBDEM_ERR_INVALID;
    }
  if (c->unitTime <= 0.0) {
    err = "unitTime must be positive";
    return LBDEM_ERR_INVALID;
  }
  demSolve = c->demSolve != 0;
  lbSolve = c->lbSolve != 0;
  freeSurface = c->freeSurfaceSolve != 0;
  forceField = c->forceFieldSolve != 0;
  demInitialRepeat = c->demInitialRepeat;
  // measureUnits::setComposite, src/node.cpp:512-525
  uLength = c->unitLength;
  uTime = c->unitTime;
  uDensity = c->unitDensity;
  uVolume = uLength * uLength * uLength;
  uSpeed = uLength / uTime;
  uAccel = uLength / uTime / uTime;
  uAngVel = 1.0 / uTime;
  uKinVisc = uLength * uLength / uTime;
  uDynVisc = uDensity * uLength * uLength / uTime;
  uForce = uDensity * uLength * uLength * uLength * uLength / uTime / uTime;
  uTorque = uDensity * uLength * uLength * uLength * uLength * uLength / uTime / uTime;
  // LB::latticeBoltzmannGet, src/LB.cpp:160-330
  X = int(std::floor(c->lbSizeX / uLength + 0.5));
  Y = int(std::floor(c->lbSizeY / uLength + 0.5));
  Z = int(std::floor(c->lbSizeZ / uLength + 0.5));
  if (X < 3 || Y < 3 || Z < 3) {
    err = "lattice too small";
    return LBDEM_ERR_INVALID;
  }
  const unsigned s[3] = {(unsigned)X, (unsigned)Y, (unsigned)Z};
  for (int k = 0; k < 3; ++k) physSize[k] = double(s[k]) * uLength;
  boundaryLoc[0] = Vec(0.5 * uLength, 0.0, 0.0);
  boundaryLoc[1] = Vec(double(s[0] - 1.5) * uLength, 0.0, 0.0);
  boundaryLoc[2] = Vec(0.0, 0.5 * uLength, 0.0);
  boundaryLoc[3] = Vec(0.0, double(s[1] - 1.5) * uLength, 0.0);
  boundaryLoc[4] = Vec(0.0, 0.0, 0.5 * uLength);
  boundaryLoc[5] = Vec(0.0, 0.0, double(s[2] - 1.5) * uLength);
  initDynVisc = c->initVisc / uDynVisc;
  // src/LB.cpp:240-326: rheology parameters in lattice units (turbConst is
  // not scaled); unit.Stress = Density * Length^2 / Time^2 (src/node.cpp:522)
  rheology = c->rheologyModel;
  plasticVisc = c->plasticVisc / uDynVisc;
  yieldStress = c->yieldStress / (uDensity * uLength * uLength / uTime / uTime);
  frictionCoefFluid = c->frictionCoefFluid;
  voellmyCoefficient = c->voellmyConstant / uAccel;
  turbulenceOn = c->turbulenceSolve != 0;
  turbConst = c->turbConst;
  initVelocity = Vec(c->initVelocity[0], c->initVelocity[1], c->initVelocity[2]) / uSpeed;
  lbF = Vec(c->lbF[0], c->lbF[1], c->lbF[2]) / uAccel;
  for (int k = 0; k < 6; ++k) boundary[k] = c->boundary[k];
  slipCoefficient = c->slipCoefficient;
  fluidHeight = c->fluidHeight;
  initDensity = 1.0;
  // DEM::discreteElementGet, src/DEM.cpp:17-166
  density = c->density;
  objectDensity = c->objectDensity;
  linearStiff = c->linearStiff;
  frictionCoefPart = c->frictionCoefPart;
  lubNormal = c->lubNormal;
  lubTangential = c->lubTangential;
  lubRotation = c->lubRotation;
  lubCutoff = c->lubCutoff;
  kinVisc = c->kinVisc;
  electroForce = c->electroForce;
  debyeLength = c->debyeLength;
  objWaitTime = c->objWaitTime;
  particles.resize(c->n_particles);
  for (int k = 0; k < c->n_particles; ++k) {
    const lbdem_particle_in& in = c->particles[k];
    Particle& q = particles[k];
    q.size = (unsigned)in.size;
    q.r = in.r;
    q.x0 = Vec(in.x[0], in.x[1], in.x[2]);
    q.x1 = Vec(in.v[0], in.v[1], in.v[2]);
    q.w1 = Vec(in.w[0], in.w[1], in.w[2]);
  }
  objects.resize(c->n_objects);
  for (int k = 0; k < c->n_objects; ++k) {
    const lbdem_object_in& in = c->objects[k];
    Object& o = objects[k];
    o.index = (unsigned)in.index;
    if (o.index >= (unsigned)c->n_objects) {
      err = "object index out of range";
      return LBDEM_ERR_INVALID;
    }
    o.r = in.r;
    o.x0 = Vec(in.x[0], in.x[1], in.x[2]);
    o.x1 = Vec(in.v[0], in.v[1], in.v[2]);
  }
  // LB::latticeDefinition, src/LB.cpp:85-126
  const long s0 = 1, s1 = X, s2 = (long)X * Y;
  const long nes[19] = {0,   s0,       -s0,      s1,       -s1,      s2,      -s2,
                        s0 + s1, -s0 - s1, -s0 + s1, s0 - s1, s1 + s2, -s1 - s2, -s1 + s2,
                        s1 - s2, s2 + s0, -s2 - s0, -s2 + s0, s2 - s0};
  for (int j = 0; j < 19; ++j) ne[j] = nes[j];
  demInit();
  if (lbSolve) lbInit();
  lbTime = 0;
  demTime = 0.0;
  demTimeStep = 0;
  return LBDEM_OK;
}

// DEM::discreteElementInit, src/DEM.cpp:199-357
void oracle_ctx::demInit() {
  demSize[0] = physSize[0];
  demSize[1] = freeSurface ? fluidHeight : physSize[1];
  demSize[2] = physSize[2];
  vol = freeSurface ? demSize[0] * fluidHeight * demSize[2]
                    : demSize[0] * demSize[1] * demSize[2];
  demF = lbF * uAccel;  // src/main.cpp:269
  unsigned globalIndex = 0;
  for (Particle& q : particles) {  // particle::initialize, src/elmt.cpp:27-63
    const double singleMass = 4.0 / 3.0 * density * PI * q.r * q.r * q.r;
    q.m = q.size * singleMass;
    q.dens = density;
    q.I = q.size * 2.0 / 5.0 * singleMass * q.r * q.r;
    q.x1 = Vec();
    q.w1 = Vec();
    q.particleIndex = globalIndex;
    q.FTotal = q.FRep = q.FHydro = q.FContact = q.FLub = Vec();
    q.FGrav = demF * q.m;
    q.MTotal = q.MHydro = q.MContact = q.MLub = Vec();
    ++globalIndex;
  }
  for (Object& o : objects) {
    o.m = 4.0 / 3.0 * objectDensity * PI * o.r * o.r * o.r;
    o.FGrav = demF * o.m;
    o.I = 2.0 / 5.0 * o.m * o.r * o.r;
    o._m = 1.0 / o.m;
    o._I = 1.0 / o.I;
  }
  for (Body& b : bodies) {  // src/DEM.cpp:257-266
    b.m = bodyDensity * (4.0 / 3.0) * PI * (b.r * b.r * b.r);
    b._m = 1.0 / b.m;
    b.FGrav = demF * b.m;
    b.L = b.L0;
  }
  // DEM::initializeWalls, src/DEM.cpp:405-458
  const Vec dirs[6] = {Vec(1, 0, 0), Vec(-1, 0, 0), Vec(0, 1, 0),
                       Vec(0, -1, 0), Vec(0, 0, 1), Vec(0, 0, -1)};
  unsigned idx = 0;
  walls.clear();
  for (int i = 0; i < 6; ++i) {
    if (boundary[i] >= 5 && boundary[i] <= 8) {
      Wall w;
      w.p = boundaryLoc[i];
      w.n = dirs[i];
      w.index = idx++;
      w.moving = boundary[0] == 6 || boundary[0] == 8;
      w.slip = boundary[0] == 5 || boundary[0] == 6;
      walls.push_back(w);
    }
  }
  for (Particle& q : particles) {
    q._m = 1.0 / q.m;
    q._I = 1.0 / q.I;
  }
  neighborList();
  newNeighborList = true;
  minPartRadius = 1.0e99;
  maxPartRadius = 0.0;
  meanPartRadius = 0.0;
  for (Particle& q : particles) {
    meanPartRadius += q.r;
    if (q.r > maxPartRadius) maxPartRadius = q.r;
    if (q.r < minPartRadius) minPartRadius = q.r;
  }
  if (!particles.empty()) meanPartRadius /= double(particles.size());
  deltat = uTime / double(1);
  const double averageMass =
      4.0 / 3.0 * density * PI * meanPartRadius * meanPartRadius * meanPartRadius;
  dampCoeff = std::sqrt(averageMass * linearStiff);
}

// LB::latticeBolzmannInit, src/LB.cpp:340-398
void oracle_ctx::lbInit() {
  N = (size_t)X * Y * Z;
  t.assign(N, 0);
  p.assign(N, 0);
  hasnode.assign(N, 0);
  solid.assign(N, 0);
  f.assign(19 * N, 0.0);
  fs.assign(19 * N, 0.0);
  n.assign(N, 0.0);
  ux.assign(N, 0.0);
  uy.assign(N, 0.0);
  uz.assign(N, 0.0);
  hx.assign(N, 0.0);
  hy.assign(N, 0.0);
  hz.assign(N, 0.0);
  mass.assign(N, 0.0);
  newMass.assign(N, 0.0);
  visc.assign(N, 0.0);
  // initializeLatticeBoundaries, src/LB.cpp:538-564
  for (size_t it = 0; it < N; ++it) {
    if (isWall(it)) continue;
    const unsigned x = getX(it), y = getY(it), z = getZ(it);
    int b = -1;
    if (x == 0) b = boundary[0];
    else if (x == (unsigned)X - 1) b = boundary[1];
    else if (y == 0) b = boundary[2];
    else if (y == (unsigned)Y - 1) b = boundary[3];
    else if (z == 0) b = boundary[4];
    else if (z == (unsigned)Z - 1) b = boundary[5];
    if (b >= 0) t[it] = (uint8_t)b;
  }
  // initializeTypes, src/LB.cpp:487-498
  // initializeParticleBoundaries with an empty active list: reset only
  for (size_t it = 0; it < N; ++it) {
    p[it] = 0;
    solid[it] = 0;
  }
  // initializeWallBoundaries, src/LB.cpp:713-748
  for (const Wall& w : walls) {
    const Vec wp = w.p / uLength;
    for (size_t it = 0; it < N; ++it)
      if (insidePlane(pos(it), wp, w.n)) {
        solid[it] = w.index;
        t[it] = w.slip ? (w.moving ? 6 : 5) : (w.moving ? 8 : 7);
      }
  }
  // initializeObjectBoundaries, src/LB.cpp:751-795
  objectNodes.clear();
  for (const Object& o : objects) {
    const Vec c = o.x0 / uLength;
    const double r = o.r / uLength;
    for (size_t it = 0; it < N; ++it)
      if (insideSphere(pos(it), c, r)) {
        solid[it] = o.index;
        t[it] = 12;
      }
  }
  for (size_t ip = 0; ip < N; ++ip) {
    if (t[ip] != 12) continue;
    createNode(ip);
    const Object& o = objects[solid[ip]];
    if (insideSphere(pos(ip), o.x0 / uLength, o.r / uLength)) {
      initialize(ip, initDensity, o.x1 / uSpeed, 0.0, 0.0, Vec());
      objectNodes.push_back((unsigned)ip);
    }
  }
  // initializeInterface, src/LB.cpp:974-992
  if (freeSurface) {
    const double h = fluidHeight / uLength;
    for (size_t it = 0; it < N; ++it)
      if (getY(it) > h && t[it] == 0) t[it] = 2;
  }
  // initializeVariables, src/LB.cpp:1042-1096
  for (size_t it = 0; it < N; ++it) {
    if (t[it] == 0) {
      createNode(it);
      for (int j = 1; j < 19; ++j)
        if (t[link(it, j)] == 2) {
          t[it] = 3;
          break;
        }
    }
    if (t[it] == 0)
      initialize(it, initDensity, initVelocity, initDensity, initDynVisc, lbF);
    else if (t[it] == 3)
      initialize(it, initDensity, initVelocity, 0.5 * initDensity, initDynVisc, lbF);
  }
  // initializeWalls, src/LB.cpp:1140-1176
  for (size_t it = 0; it < N; ++it)
    if (isWall(it)) {
      createNode(it);
      initialize(it, initDensity, Vec(), 0.0, 0.0, Vec());
    }
  initializeLists();
  cleanLists();
}

// ==== lists ================================================================

// LB::initializeLists, src/LB.cpp:1011-1040
void oracle_ctx::initializeLists() {
  fluidNodes.clear();
  particleNodes.clear();
  interfaceNodes.clear();
  for (size_t it = 0; it < N; ++it) {
    if (t[it] == 0) fluidNodes.push_back((unsigned)it);
    else if (t[it] == 3) interfaceNodes.push_back((unsigned)it);
    if (p[it]) particleNodes.push_back((unsigned)it);
  }
}

// LB::cleanLists, src/LB.cpp:1181-1259
void oracle_ctx::cleanLists() {
  auto sortUnique = [](std::vector<unsigned>& v) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  };
  sortUnique(fluidNodes);
  sortUnique(interfaceNodes);
  sortUnique(particleNodes);
  sortUnique(objectNodes);
  activeNodes.clear();
  activeNodes.insert(activeNodes.end(), fluidNodes.begin(), fluidNodes.end());
  activeNodes.insert(activeNodes.end(), interfaceNodes.begin(), interfaceNodes.end());
  std::sort(activeNodes.begin(), activeNodes.end());
  // backward erase loop (index 0 is never tested, as in the reference)
  for (long ind = (long)activeNodes.size() - 1; ind > 0; --ind) {
    const unsigned i = activeNodes[ind], j = activeNodes[ind - 1];
    if (t[i] == 2 || t[i] == 12 || !hasnode[i] || i == j)
      activeNodes.erase(activeNodes.begin() + ind);
  }
}

// ==== coupling step, src/LB.cpp:432-467 ===================================

void oracle_ctx::couplingStep() {
  updateObjectBoundaries();
  if (newNeighborList) {
    updateIndices();
    newNeighborList = false;
  }
  findNewActive();
  // findNewSolid (src/LB.cpp:2032-2100) never appends a node: its `break`
  // leaves the k loop before the append block is reached.
}

// LB::updateObjectBoundaries + findNewActiveObject, src/LB.cpp:797-943
void oracle_ctx::updateObjectBoundaries() {
  // findNewActiveObject, src/LB.cpp:846-943
  if (!objects.empty()) {
    const Object& o0 = objects[0];  // objectIndex hard-coded 0, :870
    const Vec c0 = o0.x0 / uLength;
    const double r0 = o0.r / uLength;
    for (size_t ip = 0; ip < objectNodes.size(); ++ip) {
      const size_t index = objectNodes[ip];
      bool surroundedGas = true;
      for (int j = 1; j < 19; ++j)
        if (t[link(index, j)] == 0) {
          surroundedGas = false;
          break;
        }
      bool newActive = !insideSphere(pos(index), c0, r0);
      if (newActive && surroundedGas) {
        t[index] = 2;
        hasnode[index] = 0;
        newActive = false;
      }
      if (newActive) {
        createNode(index);
        t[index] = 0;
        for (int j = 1; j < 19; ++j)
          if (t[link(index, j)] == 2) {
            t[index] = 3;
            break;
          }
        if (t[index] == 0)
          initialize(index, initDensity, initVelocity, initDensity, initDynVisc, lbF);
        else
          initialize(index, initDensity, Vec(), 0.5 * initDensity, initDynVisc, lbF);
      }
    }
  }
  objectNodes.clear();
  for (const Object& o : objects) {
    const Vec c = o.x0 / uLength;
    const double r = o.r / uLength;
    for (size_t it = 0; it < N; ++it)
      if (insideSphere(pos(it), c, r)) {
        solid[it] = o.index;
        t[it] = 12;
      }
  }
  for (size_t ip = 0; ip < N; ++ip) {
    if (t[ip] != 12) continue;
    createNode(ip);
    const Object& o = objects[solid[ip]];
    if (insideSphere(pos(ip), o.x0 / uLength, o.r / uLength)) {
      initialize(ip, initDensity, o.x1 / uSpeed, 0.0, 0.0, Vec());
      objectNodes.push_back((unsigned)ip);
    }
  }
}

// LB::updateIndices -> initializeParticleBoundaries + initializeLists,
// src/LB.cpp:1875-1899, 683-711
// The reference loops every particle over the whole active list; visiting
// only the active-list nodes of each particle's bounding box flags the same
// nodes with the same (last particle wins) indices.
void oracle_ctx::updateIndices() {
  for (size_t it = 0; it < N; ++it) {
    p[it] = 0;
    solid[it] = 0;
  }
  std::vector<uint8_t> inList(N, 0);
  for (unsigned index : activeNodes) inList[index] = 1;
  for (const Particle& q : particles) {
    const Vec c = q.x0 / uLength;
    const double r = q.r / uLength;
    const int lo[3] = {std::max(0, (int)std::floor(c.x - r) - 1), std::max(0, (int)std::floor(c.y - r) - 1),
                       std::max(0, (int)std::floor(c.z - r) - 1)};
    const int hi[3] = {std::min(X - 1, (int)std::ceil(c.x + r) + 1),
                       std::min(Y - 1, (int)std::ceil(c.y + r) + 1),
                       std::min(Z - 1, (int)std::ceil(c.z + r) + 1)};
    for (int z = lo[2]; z <= hi[2]; ++z)
      for (int y = lo[1]; y <= hi[1]; ++y)
        for (int x = lo[0]; x <= hi[0]; ++x) {
          const size_t index = (size_t)x + (size_t)y * X + (size_t)z * X * Y;
          if (inList[index] && insideSphere(pos(index), c, r)) {
            p[index] = 1;
            solid[index] = q.particleIndex;
          }
        }
  }
  initializeLists();
}

// LB::findNewActive, src/LB.cpp:1980-2029 (including the loop-exiting break)
void oracle_ctx::findNewActive() {
  std::vector<unsigned> popUp;
  for (size_t ip = 0; ip < particleNodes.size(); ++ip) {
    const unsigned index = particleNodes[ip];
    if (solid[index] >= particles.size()) {
      err = "particle node with out-of-range solid index";
      return;
    }
    const Particle& q = particles[solid[index]];
    if (insideSphere(pos(index), q.x0 / uLength, q.r / uLength)) break;
    popUp.push_back(index);
    p[index] = 0;
    solid[index] = 0;
  }
  for (unsigned u : popUp)
    for (long ind = (long)particleNodes.size() - 1; ind >= 0; --ind)
      if (particleNodes[ind] == u) particleNodes.erase(particleNodes.begin() + ind);
}

// ==== LB step, src/LB.cpp:400-418 =========================================

void oracle_ctx::lbStep() {
  initializeLists();
  cleanLists();
  // reconstruction, :1261-1299 (independent per node: threaded)
  const long na = (long)activeNodes.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < na; ++i) reconstruct(activeNodes[i]);
  computeHydroForces();
  collision();
  streaming();
}

// LB::computeHydroForces, src/LB.cpp:1901-1978
void oracle_ctx::computeHydroForces() {
  for (Particle& q : particles) {
    q.FHydro = Vec();
    q.MHydro = Vec();
    q.fluidVolume = 0.0;
    for (double& s : q.SHydro) s = 0.0;
  }
  for (unsigned index : activeNodes) {
    hx[index] = hy[index] = hz[index] = 0.0;
    if (!p[index]) continue;
    if (solid[index] >= particles.size()) {
      err = "active particle node with out-of-range solid index";
      return;
    }
    Particle& q = particles[solid[index]];
    const Vec radius = pos(index) - q.x0 / uLength;
    const Vec localVel = q.x1 / uSpeed + cross(q.w1, radius) / uAngVel;
    const double lf = mass[index] / n[index];
    const Vec diffVel = lf * (U(index) - localVel);
    const Vec h = H(index) + (-1.0 * diffVel);
    hx[index] = h.x;
    hy[index] = h.y;
    hz[index] = h.z;
    q.fluidVolume += mass[index];
    q.FHydro += 1.0 * diffVel;
    q.MHydro += 1.0 * cross(radius, diffVel);
    const double r[3] = {radius.x, radius.y, radius.z};
    const double d[3] = {diffVel.x, diffVel.y, diffVel.z};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) q.SHydro[3 * a + b] += 1.0 * r[a] * uLength * d[b] * uForce;
  }
  for (Particle& q : particles) {
    q.FHydro *= uForce;
    q.MHydro *= uTorque;
    q.fluidVolume *= uVolume;
  }
}

// LB::collision + node::shiftVelocity/solveCollision/addForce,
// src/LB.cpp:1301-1332, src/node.cpp:95-207
void oracle_ctx::collision() {
  if (!forceField) lbF = Vec();
  const long na = (long)activeNodes.size();
#pragma omp parallel for schedule(static)
  for (long ia = 0; ia < na; ++ia) {
    const unsigned index = activeNodes[ia];
    double feq[19];
    const Vec total = lbF + H(index);
    setU(index, U(index) + 0.5 * total / n[index]);
    computeEquilibrium(index, feq);
    if (rheology != LBDEM_NEWTONIAN || turbulenceOn) computeApparentViscosity(index, feq);
    const double omega = 1.0 / (0.5 + 3.0 * visc[index]);
    for (int j = 0; j < 19; ++j) F(j, index) += omega * (feq[j] - F(j, index));
    const double omegaf = 1.0 - 1.0 / (1.0 + 6.0 * visc[index]);
    const Vec u = U(index);
    for (int j = 0; j < 19; ++j) {
      const double vu = dot(u, vdir(j));
      const Vec vmu = vdir(j) - u;
      const Vec forcePart = 9.0 * vu * vdir(j) + 3.0 * vmu;
      F(j, index) += omegaf * COEFF[j] * dot(forcePart, total);
    }
  }
}

// LB::streaming, src/LB.cpp:1334-1544
void oracle_ctx::streaming() {
  const double S1 = slipCoefficient, S2 = 1.0 - slipCoefficient;
  double sp[19];
  for (int j = 0; j < 19; ++j) sp[j] = initDensity * COEFF[j];
  const double BBCoeff = 2.0 * 3.0;
  double extraMass = 0.0;
  for (Wall& w : walls) w.FHydro = Vec();
  for (Object& o : objects) {
    o.FHydro = Vec();
    o.MHydro = Vec();
  }
  const long na = (long)activeNodes.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < na; ++i)
    for (int j = 0; j < 19; ++j) FS(j, activeNodes[i]) = F(j, activeNodes[i]);
  for (unsigned it : activeNodes) {
    for (int j = 1; j < 19; ++j) {
      const size_t lk = (size_t)link(it, j);
      const uint8_t tl = t[lk];
      const int o = OPP[j];
      if (tl == 0 || tl == 3) {
        F(o, it) = FS(o, lk);
      } else if (tl == 2) {
        const Vec u = U(it);
        const double usq = norm2(u);
        const double vuj = dot(u, vdir(j));
        F(o, it) = -FS(j, it) + COEFF[j] * initDensity * (2.0 + 9.0 * (vuj * vuj) - 3.0 * usq);
      } else if (tl == 11) {
        F(o, it) = FS(j, it);
      } else if (tl == 8) {
        const Vec vel = U(lk);
        const double BBi = BBCoeff * n[it] * COEFF[j] * dot(vel, vdir(j));
        if (solid[lk] < walls.size()) walls[solid[lk]].FHydro += bounceBackForce(it, j, sp, BBi);
        F(o, it) = FS(j, it) - BBi;
        extraMass += BBi * mass[it];
      } else if (tl == 7) {
        if (solid[lk] < walls.size()) walls[solid[lk]].FHydro += bounceBackForce(it, j, sp, 0.0);
        F(o, it) = FS(j, it);
      } else if (tl == 12) {
        const Vec vel = U(lk);
        const double BBi = BBCoeff * n[it] * COEFF[j] * dot(vel, vdir(j));
        // An object node whose solid index was overwritten by a particle
        // index (updateIndices runs on the pre-coupling active list) makes
        // the reference index past the object vector; the force is dropped.
        if (solid[lk] < objects.size()) {
          Object& ob = objects[solid[lk]];
          const Vec BBforce = bounceBackForce(it, j, sp, BBi);
          const Vec rad = pos(lk) - ob.x0 / uLength;
          ob.FHydro += BBforce;
          ob.MHydro += cross(rad, BBforce);
        }
        F(o, it) = FS(j, it) - BBi;
        extraMass += BBi * mass[it];
      } else if (tl == 5 || tl == 6) {
        double BBi = 0.0;
        if (tl == 6) BBi = BBCoeff * n[it] * COEFF[j] * dot(U(lk), vdir(j));
        if (j > 6) {
          const size_t c1 = (size_t)link(it, (int)SLIP1C[j]);
          const size_t c2 = (size_t)link(it, (int)SLIP2C[j]);
          const bool a1 = isActive(c1), a2 = isActive(c2);
          if (a1 && !a2) {
            F(o, it) = tl == 5 ? S1 * FS(SLIP1[j], c1) + S2 * FS(j, it)
                               : S1 * FS(SLIP1[j], c1) + S2 * (FS(j, it) - BBi);
            if (tl == 6) extraMass += S2 * mass[it] * BBi;
          } else if (!a1 && a2) {
            F(o, it) = tl == 5 ? S1 * FS(SLIP2[j], c2) + S2 * FS(j, it)
                               : S1 * FS(SLIP2[j], c2) + S2 * (FS(j, it) - BBi);
            if (tl == 6) extraMass += S2 * mass[it] * BBi;
          } else {
            F(o, it) = tl == 5 ? FS(j, it) : FS(j, it) - BBi;
            if (tl == 6) extraMass += mass[it] * BBi;
          }
        } else {
          F(o, it) = tl == 5 ? FS(j, it) : FS(j, it) - BBi;
          if (tl == 6) extraMass += mass[it] * BBi;
        }
      } else {
        err = "TYPE ERROR in streaming";
      }
    }
  }
  redistributeMass(extraMass);
  for (Wall& w : walls) w.FHydro *= uForce;
  for (Object& o : objects) {
    o.FHydro *= uForce;
    o.MHydro *= uTorque;
  }
}

// LB::redistributeMass, src/LB.cpp:1844-1852
void oracle_ctx::redistributeMass(double massSurplus) {
  const double addMass = massSurplus / interfaceNodes.size();
  for (unsigned it : interfaceNodes) mass[it] += addMass;
}

// ==== free-surface step, src/LB.cpp:422-430 ================================

void oracle_ctx::fsStep() {
  updateMass();
  updateInterface();
  cleanLists();
}

// LB::updateMass, src/LB.cpp:1548-1639
void oracle_ctx::updateMass() {
  for (unsigned it : interfaceNodes) newMass[it] = mass[it];
  for (unsigned index : interfaceNodes) {
    double deltaMass = 0.0;
    for (int j = 1; j < 19; ++j) {
      const size_t lk = (size_t)link(index, j);
      const uint8_t tl = t[lk];
      if (tl == 3) {
        const double averageMass = 0.5 * (mass[lk] + mass[index]);
        deltaMass += averageMass * massStream(index, j);
      } else if (tl == 0) {
        const double averageMass = 1.0;
        deltaMass += averageMass * massStream(index, j);
      } else if (tl == 8 || tl == 12 || tl == 9) {
        const double averageMass = 1.0 * mass[index];
        deltaMass += averageMass * massStream(index, j);
      } else if (tl == 6) {
        double averageMass = 0.0;
        if (j > 6) {
          const bool a1 = isActive((size_t)link(index, (int)SLIP1C[j]));
          const bool a2 = isActive((size_t)link(index, (int)SLIP2C[j]));
          if ((a1 && !a2) || (!a1 && a2))
            averageMass += 1.0 * (1.0 - slipCoefficient) * mass[index];
          else
            averageMass += 1.0 * mass[index];
        } else {
          averageMass = 1.0 * mass[index];
        }
        deltaMass += averageMass * massStream(index, j);
      }
    }
    newMass[index] += deltaMass;
  }
  for (unsigned it : fluidNodes) mass[it] = n[it];
  for (unsigned it : interfaceNodes) mass[it] = newMass[it];
}

// LB::updateInterface and its helpers, src/LB.cpp:1641-1842
void oracle_ctx::updateInterface() {
  double massSurplus = 0.0;
  std::vector<unsigned> filled, emptied, newIf;
  // findInterfaceMutants, :1669-1698
  for (long ind = (long)interfaceNodes.size() - 1; ind >= 0; --ind) {
    const unsigned i = interfaceNodes[ind];
    if (mass[i] > n[i]) {
      filled.push_back(i);
      t[i] = 0;
      fluidNodes.push_back(i);
      interfaceNodes.erase(interfaceNodes.begin() + ind);
    } else if (mass[i] < 0.0) {
      emptied.push_back(i);
      t[i] = 2;
      interfaceNodes.erase(interfaceNodes.begin() + ind);
    }
  }
  // smoothenInterface, :1700-1749
  for (unsigned index : filled)
    for (int j = 1; j < 19; ++j) {
      const size_t lk = (size_t)link(index, j);
      if (t[lk] == 2) {
        t[lk] = 3;
        newIf.push_back((unsigned)lk);
        createNode(lk);
        initialize(lk, initDensity, U(index), 0.01 * initDensity, visc[index], H(index) + lbF);
        massSurplus -= 0.01 * initDensity;
      }
    }
  for (unsigned index : emptied)
    for (int j = 0; j < 19; ++j) {
      const size_t lk = (size_t)link(index, j);
      if (t[lk] == 0) {
        t[lk] = 3;
        newIf.push_back((unsigned)lk);
        mass[lk] = 0.99 * n[lk];
        massSurplus += 0.01 * n[lk];
        for (long ind = (long)fluidNodes.size() - 1; ind >= 0; --ind)
          if (fluidNodes[ind] == lk) fluidNodes.erase(fluidNodes.begin() + ind);
      }
    }
  // updateMutants, :1751-1790
  auto isNew = [&](unsigned i) {
    for (unsigned k : newIf)
      if (k == i) return true;
    return false;
  };
  for (unsigned i : emptied)
    if (!isNew(i)) {
      massSurplus += mass[i];
      hasnode[i] = 0;
    }
  for (unsigned i : filled)
    if (!isNew(i)) {
      massSurplus += mass[i] - n[i];
      mass[i] = n[i];
    }
  for (unsigned i : newIf) interfaceNodes.push_back(i);
  // removeIsolated, :1792-1842
  for (long ind = (long)interfaceNodes.size() - 1; ind >= 0; --ind) {
    const unsigned i = interfaceNodes[ind];
    bool surroundedFluid = true;
    for (int j = 1; j < 19; ++j)
      if (t[link(i, j)] == 2) {
        surroundedFluid = false;
        break;
      }
    if (surroundedFluid) {
      massSurplus += mass[i] - n[i];
      mass[i] = n[i];
      t[i] = 0;
      interfaceNodes.erase(interfaceNodes.begin() + ind);
      fluidNodes.push_back(i);
    }
  }
  for (long ind = (long)interfaceNodes.size() - 1; ind >= 0; --ind) {
    const unsigned i = interfaceNodes[ind];
    bool surroundedGas = true;
    for (int j = 1; j < 19; ++j)
      if (t[link(i, j)] == 0) {
        surroundedGas = false;
        break;
      }
    if (surroundedGas) {
      massSurplus += mass[i];
      interfaceNodes.erase(interfaceNodes.begin() + ind);
      t[i] = 2;
      hasnode[i] = 0;
    }
  }
  redistributeMass(massSurplus);
}

// ==== DEM step, src/DEM.cpp:359-401 ========================================

void oracle_ctx::demStep() {
  ++demTimeStep;
  demTime += deltat;
  // evalMaxDisp, :460-470
  double maxVel = 0.0;
  for (const Particle& q : particles)
    if (norm2(q.x1) > maxVel) maxVel = norm2(q.x1);
  maxVel = std::sqrt(maxVel);
  maxDisp += maxVel * deltat;
  if (maxDisp > 0.05) {
    maxDisp = 0.0;
    neighborList();
    newNeighborList = true;
  }
  evaluateForces();
  integration();
}

// DEM::neighborList, src/DEM.cpp:473-652
void oracle_ctx::neighborList() {
  ++rebuilds;
  const int num = (int)particles.size();
  for (Particle& q : particles) {
    std::memcpy(q._list, q.list, sizeof(q.list));
    std::memcpy(q._xix, q.xix, sizeof(q.xix));
    std::memcpy(q._xiy, q.xiy, sizeof(q.xiy));
    std::memcpy(q._xiz, q.xiz, sizeof(q.xiz));
  }
  double r_max = 0.0;
  for (Particle& q : particles) {
    r_max = dmax(r_max, q.r);
    q.list[0] = 0;
    q.xix[0] = q.xiy[0] = q.xiz[0] = 0.0;
  }
  double cut = 2.0 * r_max + 2.0;
  const int nlx = (int)(demSize[0] / cut), nly = (int)(demSize[1] / cut),
            nlz = (int)(demSize[2] / cut);
  auto append = [&](int n1, int n2) {
    Particle& a = particles[n1];
    Particle& b = particles[n2];
    if (a.list[0] + 1 >= MAX_N || b.list[0] + 1 >= MAX_N) {
      err = "neighbour list overflow";
      return false;
    }
    a.list[0]++;
    b.list[0]++;
    a.xix[0] += 1.0;
    a.xiy[0] += 1.0;
    a.xiz[0] += 1.0;
    b.xix[0] += 1.0;
    b.xiy[0] += 1.0;
    b.xiz[0] += 1.0;
    a.list[a.list[0]] = n2;
    b.list[b.list[0]] = n1;
    return true;
  };
  if (std::min(nlx, nly) < 3) {  // direct sum, :515-554
    for (int n1 = 1; n1 < num; ++n1)
      for (int n2 = 0; n2 < n1; ++n2) {
        Particle& a = particles[n1];
        Particle& b = particles[n2];
        const double x12 = n_image(a.x0.x - b.x0.x, demSize[0]);
        const double y12 = n_image(a.x0.y - b.x0.y, demSize[1]);
        const double z12 = n_image(a.x0.z - b.x0.z, demSize[2]);
        const double r12 = x12 * x12 + y12 * y12 + z12 * z12;
        const double c = a.r + b.r + 2.0;
        if (r12 <= c * c) {
          if (!append(n1, n2)) return;
          const int ca = a.list[0], cb = b.list[0];
          a.xix[ca] = b.xix[cb];
          b.xix[cb] = a.xix[ca];
          a.xiy[ca] = b.xiy[cb];
          b.xiy[cb] = a.xiy[ca];
          a.xiz[ca] = b.xiz[cb];
          b.xiz[cb] = a.xiz[ca];
        }
      }
  } else {  // cell structure, :555-628
    const long ncell = (long)nlx * nly * nlz;
    if (ncell > 100000) {
      err = "cell list overflow";
      return;
    }
    cellList.assign((size_t)ncell * (MAX_N + 1), 0);
    auto cell = [&](long l, int k) -> int& { return cellList[(size_t)l * (MAX_N + 1) + k]; };
    for (int n1 = 0; n1 < num; ++n1) {
      Particle& a = particles[n1];
      const int lx = (int)(box(a.x0.x / demSize[0], 1) * nlx);
      const int ly = (int)(box(a.x0.y / demSize[1], 1) * nly);
      const int lz = (int)(box(a.x0.z / demSize[2], 1) * nlz);
      const long l1 = (long)lx * nly * nlz + (long)ly * nlz + lz;
      if (!(std::isfinite(a.x0.x) && std::isfinite(a.x0.y) && std::isfinite(a.x0.z)) ||
          lx < 0 || lx >= nlx || ly < 0 || ly >= nly || lz < 0 || lz >= nlz) {
        err = "particle " + std::to_string(n1) + " outside the cell grid (non-finite position)";
        return;
      }
      if (cell(l1, 0) >= MAX_N) {
        err = "cell occupancy overflow";
        return;
      }
      cell(l1, 0)++;
      cell(l1, cell(l1, 0)) = n1;
      a.list[0] = 0;
      a.xix[0] = a.xiy[0] = a.xiz[0] = 0.0;
    }
    for (int lx1 = 0; lx1 < nlx; lx1++)
      for (int ly1 = 0; ly1 < nly; ly1++)
        for (int lz1 = 0; lz1 < nlz; lz1++)
          for (int lx2 = lx1 - 1; lx2 <= lx1 + 1; lx2++)
            for (int ly2 = ly1 - 1; ly2 <= ly1 + 1; ly2++)
              for (int lz2 = lz1 - 1; lz2 <= lz1 + 1; lz2++) {
                const long l1 = (long)lx1 * nly * nlz + (long)ly1 * nlz + lz1;
                const long l2 = (long)((lx2 + nlx) % nlx) * nly * nlz +
                                (long)((ly2 + nly) % nly) * nlz + (lz2 + nlz) % nlz;
                for (int a1 = 1; a1 <= cell(l1, 0); a1++)
                  for (int a2 = 1; a2 <= cell(l2, 0); a2++) {
                    const int n1 = cell(l1, a1), n2 = cell(l2, a2);
                    if (n2 < n1) {
                      Particle& a = particles[n1];
                      Particle& b = particles[n2];
                      const double x12 = n_image(a.x0.x - b.x0.x, demSize[0]);
                      const double y12 = n_image(a.x0.y - b.x0.y, demSize[1]);
                      const double z12 = n_image(a.x0.z - b.x0.z, demSize[2]);
                      const double r12 = x12 * x12 + y12 * y12 + z12 * z12;
                      const double c = a.r + b.r + 2.0;
                      if (r12 <= c * c)
                        if (!append(n1, n2)) return;
                    }
                  }
              }
  }
  // tangential history carry-over, :633-651
  for (Particle& q : particles)
    for (int nn = 1; nn <= q.list[0]; nn++) {
      const int k = q.list[nn];
      for (int l = 1; l <= q._list[0]; l++)
        if (q._list[l] == k) {
          q.xix[nn] = q._xix[l];
          q.xiy[nn] = q._xiy[l];
          q.xiz[nn] = q._xiz[l];
        }
    }
}

// DEM::evaluateForces, src/DEM.cpp:655-796
void oracle_ctx::evaluateForces() {
  for (Particle& q : particles) {
    q.FTotal = q.MTotal = q.FContact = q.MContact = Vec();
    q.FLub = q.MLub = q.FRep = Vec();
  }
  for (Object& o : objects) {
    o.FTotal = o.FContact = o.FLub = o.FSpring = Vec();
    o.MTotal = o.MContact = o.MLub = Vec();
  }
  for (Wall& w : walls) w.FTotal = w.FContact = w.FLub = w.FRep = Vec();
  for (Body& b : bodies) b.FTotal = b.FSpring = Vec();
  if ((int)demTimeStep >= objWaitTime) {
    if (!bodies.empty()) bodyObjectInteraction();
    particleLubrication();
    wallLubrication();
    objectContact();
    objectLubrication();
  } else {
    wallContact(true);
  }
  particleContact();
  particleElectro();
  wallContact(false);
  for (Particle& q : particles) {
    q.FTotal += q.FHydro + q.FContact + q.FLub + q.FGrav + q.FRep;
    q.MTotal += q.MHydro + q.MContact + q.MLub;
  }
  for (Wall& w : walls) w.FTotal += w.FHydro + w.FContact + w.FLub + w.FRep;
  if ((int)demTimeStep <= objWaitTime)
    for (Particle& q : particles) q.FGrav = Vec();
  for (Object& o : objects) {
    o.FTotal += o.FHydro + o.FContact + o.FLub + o.FGrav + o.FSpring;
    o.MTotal += o.MHydro + o.MContact + o.MLub;
  }
  for (Body& b : bodies) b.FTotal += b.FGrav + b.FSpring;
}

// DEM::bodyObjectInteraction, src/DEM.cpp:798-869: a spring along y between
// every body and every impactor (nonLinType 0-4)
void oracle_ctx::bodyObjectInteraction() {
  for (Body& bd : bodies)
    for (Object& ob : objects) {
      double fs = 0.0, fdo = 0.0, fdb = 0.0;
      bd.L = bd.x0.y - ob.x0.y;
      const Vec r = bd.x0 - ob.x0;
      const double rn = std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
      const double ny = r.y / rn;
      const double del = bd.L0 - bd.L;
      const double bodyDamp = 2.0 * std::sqrt(bd.m * bd.k) * springDamp;
      const double objDamp = 2.0 * std::sqrt(ob.m * bd.k) * springDamp;
      const double sigma = bd.r;
      if (nonLinType == 0) {
        fs = bd.k * del * ny;
      } else if (nonLinType == 1) {
        fs = (bd.k * del) * ny;
        fdo = -ob.x1.y * objDamp;
        fdb = -bd.x1.y * bodyDamp;
      } else if (nonLinType == 2) {
        fs = (bd.k * del + k13 * bd.k * (del * del * del)) * ny;
        fdo = -ob.x1.y * objDamp;
        fdb = -bd.x1.y * bodyDamp;
      } else if (nonLinType == 3) {
        fs = (bd.k * del + (24.0 * epsilon / rn) * 2.0 * std::pow(sigma / rn, 12.0)) * ny;
        fdo = -ob.x1.y * objDamp;
        fdb = -bd.x1.y * bodyDamp;
      } else if (nonLinType == 4) {
        const double wcacut = std::pow(2.0, 1.0 / 6.0) * sigma;
        if (rn <= wcacut)
          fs = (bd.k * del + (24.0 * epsilon / rn) *
                                 (2.0 * std::pow(sigma / rn, 12.0) - std::pow(sigma / rn, 6.0))) *
               ny;
        else
          fs = (bd.k * del) * ny;
        fdo = -ob.x1.y * objDamp;
        fdb = -bd.x1.y * bodyDamp;
      }
      ob.FSpring.y -= fs;
      bd.FSpring.y += fs;
      ob.FSpring.y += fdo;
      bd.FSpring.y += fdb;
    }
}

// DEM::calculateParticleContactForces, src/DEM.cpp:1487-1791
void oracle_ctx::particleContact() {
  const double k = linearStiff, c = dampCoeff;
  for (int n1 = 0; n1 < (int)particles.size(); n1++) {
    Particle& a = particles[n1];
    for (int s = 1; s <= a.list[0]; s++) {
      const int n2 = a.list[s];
      if (n2 >= n1) continue;
      Particle& b = particles[n2];
      const double rad = 0.5 * (a.r + b.r);
      const double x12 = a.x0.x - b.x0.x, y12 = a.x0.y - b.x0.y, z12 = a.x0.z - b.x0.z;
      const double r12 = std::sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      const double urx = a.x1.x - b.x1.x, ury = a.x1.y - b.x1.y, urz = a.x1.z - b.x1.z;
      const double nx = x12 / r12, ny = y12 / r12, nz = z12 / r12;
      const double gn = urx * nx + ury * ny + urz * nz;
      const double mu = frictionCoefPart;
      const double del = 2 * rad - r12;
      double fnx, fny, fnz, ftx, fty, ftz;
      if (del > 0.0) {
        if (mu != 0.0) {
          const double ox = a.r * a.w1.x + b.r * b.w1.x;
          const double oy = a.r * a.w1.y + b.r * b.w1.y;
          const double oz = a.r * a.w1.z + b.r * b.w1.z;
          const double vx = urx + ny * oz - nz * oy - gn * nx;
          const double vy = ury + nz * ox - nx * oz - gn * ny;
          const double vz = urz + nx * oy - ny * ox - gn * nz;
          const double xi12 = a.xix[s] * nx + a.xiy[s] * ny + a.xiz[s] * nz;
          a.xix[s] -= xi12 * nx;
          a.xiy[s] -= xi12 * ny;
          a.xiz[s] -= xi12 * nz;
          fnx = k * del * nx - c * gn * nx;
          fny = k * del * ny - c * gn * ny;
          fnz = k * del * nz - c * gn * nz;
          const double kt = 0.2 * k;
          const double dct = kinVisc == 0.0 ? c : 0.0;
          ftx = -kt * a.xix[s] - dct * vx;
          fty = -kt * a.xiy[s] - dct * vy;
          ftz = -kt * a.xiz[s] - dct * vz;
          const double fnn = std::sqrt(fnx * fnx + fny * fny + fnz * fnz);
          const double ftt = std::sqrt(ftx * ftx + fty * fty + ftz * ftz);
          const double fri = mu * fnn;
          const double tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
          a.xix[s] += vx * deltat;
          a.xiy[s] += vy * deltat;
          a.xiz[s] += vz * deltat;
          if (fri < ftt) {
            ftx = fri * tx;
            fty = fri * ty;
            ftz = fri * tz;
            a.xix[s] = -(1 / kt) * (ftx + dct * vx);
            a.xiy[s] = -(1 / kt) * (fty + dct * vy);
            a.xiz[s] = -(1 / kt) * (ftz + dct * vz);
          }
        } else {
          fnx = k * del * nx - c * gn * nx;
          fny = k * del * ny - c * gn * ny;
          fnz = k * del * nz - c * gn * nz;
          ftx = fty = ftz = 0.0;
        }
      } else {
        fnx = fny = fnz = ftx = fty = ftz = 0.0;
        a.xix[s] = a.xiy[s] = a.xiz[s] = 0.0;
      }
      const double dfx = fnx + ftx, dfy = fny + fty, dfz = fnz + ftz;
      const double dtx = fty * nz - ftz * ny;
      const double dty = ftz * nx - ftx * nz;
      const double dtz = ftx * ny - fty * nx;
      a.FContact.x += dfx;
      a.FContact.y += dfy;
      a.FContact.z += dfz;
      b.FContact.x -= dfx;
      b.FContact.y -= dfy;
      b.FContact.z -= dfz;
      a.MContact.x += a.r * dtx;
      a.MContact.y += a.r * dty;
      a.MContact.z += a.r * dtz;
      b.MContact.x += b.r * dtx;
      b.MContact.y += b.r * dty;
      b.MContact.z += b.r * dtz;
    }
  }
}

// DEM::calculateParticleElectroForces, src/DEM.cpp:1404-1484
void oracle_ctx::particleElectro() {
  for (int n1 = 0; n1 < (int)particles.size(); n1++) {
    Particle& a = particles[n1];
    for (int s = 1; s <= a.list[0]; s++) {
      const int n2 = a.list[s];
      if (n2 >= n1) continue;
      Particle& b = particles[n2];
      const double rad = 0.5 * (a.r + b.r);
      const double x12 = a.x0.x - b.x0.x, y12 = a.x0.y - b.x0.y, z12 = a.x0.z - b.x0.z;
      const double r12 = std::sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      const double nx = x12 / r12, ny = y12 / r12, nz = z12 / r12;
      const double del = 2 * rad - r12;
      double frx, fry, frz;
      if (del <= 0.0) {
        frx = electroForce * std::exp(del / debyeLength) * nx;
        fry = electroForce * std::exp(del / debyeLength) * ny;
        frz = electroForce * std::exp(del / debyeLength) * nz;
      } else {
        frx = electroForce * nx;
        fry = electroForce * ny;
        frz = electroForce * nz;
      }
      a.FRep.x += frx;
      a.FRep.y += fry;
      a.FRep.z += frz;
      b.FRep.x -= frx;
      b.FRep.y -= fry;
      b.FRep.z -= frz;
    }
  }
}

// DEM::calculateParticleLubricationForces, src/DEM.cpp:2302-2521
void oracle_ctx::particleLubrication() {
  const double lub_N = lubNormal, lub_T = lubTangential, lub_R = lubRotation;
  for (int n1 = 0; n1 < (int)particles.size(); n1++) {
    Particle& a = particles[n1];
    for (int s = 1; s <= a.list[0]; s++) {
      const int n2 = a.list[s];
      if (n2 >= n1) continue;
      Particle& b = particles[n2];
      const double cut = lubCutoff;
      const double rad = 0.5 * (a.r + b.r);
      double x12 = a.x0.x - b.x0.x, y12 = a.x0.y - b.x0.y, z12 = a.x0.z - b.x0.z;
      const double r12 = std::sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      const double umx = a.x1.x - b.x1.x, umy = a.x1.y - b.x1.y, umz = a.x1.z - b.x1.z;
      const double w1x = a.w1.x, w1y = a.w1.y, w1z = a.w1.z;
      const double w2x = b.w1.x, w2y = b.w1.y, w2z = b.w1.z;
      const double dr = r12 - 2.0 * rad;
      const double h = dmax(dr, cut);
      if (!(dr < dmax(cut, dmax(lub_N, dmax(lub_T, lub_R))))) continue;
      const double alpha = PI * kinVisc * rad * deltat;
      const double beta1 = b.r / a.r;
      const double beta2 = beta1 * beta1;
      const double beta3 = beta1 * beta2;
      const double beta4 = std::pow((1 + beta1), 4.0);
      const double beta5 = std::pow((1 + beta1), 5.0);
      double Xa, Xg1, Xg2, Ya, Yb1, Yb2, Yg1, Yg2;
      double Yc11, Yc12, Yc21, Yc22, Yh11, Yh12, Yh21, Yh22, h_c, beta;
      if (dr < dmax(cut, lub_N)) {
        Xa = 4.0 * beta2 / beta4;
        Xg1 = 12.0 * beta2 / beta5;
        Xg2 = -12.0 * beta3 / beta5;
        h_c = dmax(dr, lub_N);
        Xa *= rad / h - rad / h_c;
        Xg1 *= rad / h - rad / h_c;
        Xg2 *= rad / h - rad / h_c;
        Xa *= 6.0 * alpha;
        Xg1 *= 4.0 * alpha * rad;
        Xg2 *= 4.0 * alpha * rad;
      } else
        Xa = Xg1 = Xg2 = 0.0;
      if (dr < dmax(cut, lub_T)) {
        Ya = 8.0 * beta1 * (2.0 + beta1 + 2.0 * beta2) / (15.0 * beta4);
        Yb1 = -4.0 * beta1 * (4.0 + beta1) / (5.0 * beta4);
        Yb2 = 4.0 * beta1 * (4.0 * beta2 + beta1) / (5.0 * beta4);
        Yg1 = 2.0 * beta1 * (4.0 - beta1 + 7.0 * beta2) / (5.0 * beta5);
        Yg2 = -2.0 * beta2 * (4.0 * beta2 - beta1 + 7.0) / (5.0 * beta5);
        h_c = dmax(dr, lub_T);
        beta = alpha * std::log(h_c / h);
        Ya *= 6.0 * beta;
        Yb1 *= 4.0 * beta * rad;
        Yb2 *= 4.0 * beta * rad;
        Yg1 *= 4.0 * beta * rad;
        Yg2 *= 4.0 * beta * rad;
      } else
        Ya = Yb1 = Yb2 = Yg1 = Yg2 = 0.0;
      if (dr < dmax(cut, lub_R)) {
        Yc11 = 16.0 * beta1 / (5.0 * beta4);
        Yc12 = 4.0 * beta2 / (5.0 * beta4);
        Yc21 = 4.0 * beta2 / (5.0 * beta4);
        Yc22 = 16.0 * beta3 / (5.0 * beta4);
        Yh11 = 4.0 * beta1 * (2.0 - beta1) / (5.0 * beta5);
        Yh12 = 2.0 * beta2 * (1.0 + 7.0 * beta1) / (5.0 * beta5);
        Yh21 = 2.0 * beta2 * (beta1 + 7.0) / (5.0 * beta5);
        Yh22 = 4.0 * beta2 * (2.0 * beta2 - beta1) / (5.0 * beta5);
        h_c = dmax(dr, lub_R);
        beta = alpha * std::log(h_c / h);
        Yc11 *= 8.0 * beta * rad * rad;
        Yc12 *= 8.0 * beta * rad * rad;
        Yc21 *= 8.0 * beta * rad * rad;
        Yc22 *= 8.0 * beta * rad * rad;
        Yh11 *= 8.0 * beta * rad * rad;
        Yh21 *= 8.0 * beta * rad * rad;
        Yh12 *= 8.0 * beta * rad * rad;
        Yh22 *= 8.0 * beta * rad * rad;
      } else
        Yc11 = Yc12 = Yc21 = Yc22 = Yh11 = Yh12 = Yh21 = Yh22 = 0.0;
      (void)Xg1;
      (void)Xg2;
      (void)Yg1;
      (void)Yg2;
      (void)Yh11;
      (void)Yh12;
      (void)Yh21;
      (void)Yh22;
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
      a.FLub.x += Fx;
      a.FLub.y += Fy;
      a.FLub.z += Fz;
      b.FLub.x -= Fx;
      b.FLub.y -= Fy;
      b.FLub.z -= Fz;
      a.MLub.x += T1x;
      a.MLub.y += T1y;
      a.MLub.z += T1z;
      b.MLub.x += T2x;
      b.MLub.y += T2y;
      b.MLub.z += T2z;
    }
  }
}

// DEM::calculateWallContactForces, src/DEM.cpp:1946-2153 (fictional=false)
// DEM::calculateFictionalWallContactForces, src/DEM.cpp:2157-2296 (true)
void oracle_ctx::wallContact(bool fictional) {
  const double k = linearStiff, c = dampCoeff;
  double nwx = 0.0, nwy = 0.0, nwz = 0.0;  // function-scope, stale between iterations
  const size_t nw = fictional ? 1 : walls.size();
  for (Particle& a : particles) {
    for (size_t w = 0; w < nw; ++w) {
      const double radw = a.r;
      double x1w, y1w, z1w;
      if (fictional) {
        x1w = 0.0;
        y1w = a.x0.y - (demSize[1] - 0.3);
        z1w = 0.0;
      } else {
        const Wall& W = walls[w];
        x1w = (a.x0.x - W.p.x) * W.n.x * W.n.x;
        y1w = (a.x0.y - W.p.y) * W.n.y * W.n.y;
        z1w = (a.x0.z - W.p.z) * W.n.z * W.n.z;
      }
      const double r1w = std::sqrt(x1w * x1w + y1w * y1w + z1w * z1w);
      const double urx = a.x1.x, ury = a.x1.y, urz = a.x1.z;
      const double delw = radw - r1w;
      double fnx, fny, fnz, ftx, fty, ftz;
      if (delw > 0.0) {
        nwx = x1w / r1w;
        nwy = y1w / r1w;
        nwz = z1w / r1w;
        const double gn = urx * nwx + ury * nwy + urz * nwz;
        const double mu = frictionCoefPart;
        if (mu != 0.0) {
          const double ox = a.r * a.w1.x, oy = a.r * a.w1.y, oz = a.r * a.w1.z;
          const double vx = urx + nwy * oz - nwz * oy - gn * nwx;
          const double vy = ury + nwz * ox - nwx * oz - gn * nwy;
          const double vz = urz + nwx * oy - nwy * ox - gn * nwz;
          const double xi = a.xiw.x * nwx + a.xiw.y * nwy + a.xiw.z * nwz;
          a.xiw.x -= xi * nwx;
          a.xiw.y -= xi * nwy;
          a.xiw.z -= xi * nwz;
          fnx = k * delw * nwx - c * gn * nwx;
          fny = k * delw * nwy - c * gn * nwy;
          fnz = k * delw * nwz - c * gn * nwz;
          const double kt = 0.2 * k;
          const double dct = kinVisc == 0.0 ? c : 0.0;
          ftx = -kt * a.xiw.x - dct * vx;
          fty = -kt * a.xiw.y - dct * vy;
          ftz = -kt * a.xiw.z - dct * vz;
          const double fnn = std::sqrt(fnx * fnx + fny * fny + fnz * fnz);
          const double ftt = std::sqrt(ftx * ftx + fty * fty + ftz * ftz);
          const double fri = mu * fnn;
          const double tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
          a.xiw.x += vx * deltat;
          a.xiw.y += vy * deltat;
          a.xiw.z += vz * deltat;
          if (fri < ftt) {
            ftx = fri * tx;
            fty = fri * ty;
            ftz = fri * tz;
            a.xiw.x = -(1 / kt) * (ftx + dct * vx);
            a.xiw.y = -(1 / kt) * (fty + dct * vy);
            a.xiw.z = -(1 / kt) * (ftz + dct * vz);
          }
        } else {
          fnx = k * delw * nwx - c * gn * nwx;
          fny = k * delw * nwy - c * gn * nwy;
          fnz = k * delw * nwz - c * gn * nwz;
          ftx = fty = ftz = 0.0;
        }
      } else {
        fnx = fny = fnz = ftx = fty = ftz = 0.0;
        a.xiw = Vec();
      }
      const double dfx = fnx + ftx, dfy = fny + fty, dfz = fnz + ftz;
      const double dtx = fty * nwz - ftz * nwy;
      const double dty = ftz * nwx - ftx * nwz;
      const double dtz = ftx * nwy - fty * nwx;
      a.FContact.x += dfx;
      a.FContact.y += dfy;
      a.FContact.z += dfz;
      if (!fictional) {
        walls[w].FContact.x -= dfx;
        walls[w].FContact.y -= dfy;
        walls[w].FContact.z -= dfz;
      }
      a.MContact.x += a.r * dtx;
      a.MContact.y += a.r * dty;
      a.MContact.z += a.r * dtz;
    }
  }
}

// DEM::calculateWallLubricationForces, src/DEM.cpp:2525-2672
void oracle_ctx::wallLubrication() {
  const double lub_N = lubNormal, lub_T = lubTangential, lub_R = lubRotation;
  for (Particle& a : particles)
    for (Wall& W : walls) {
      const double cut = lubCutoff;
      const double rad = a.r;
      double x12 = (a.x0.x - W.p.x) * W.n.x * W.n.x;
      double y12 = (a.x0.y - W.p.y) * W.n.y * W.n.y;
      double z12 = (a.x0.z - W.p.z) * W.n.z * W.n.z;
      const double r12 = std::sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      const double umx = a.x1.x, umy = a.x1.y, umz = a.x1.z;
      const double w1x = a.w1.x, w1y = a.w1.y, w1z = a.w1.z;
      const double dr = r12 - rad;
      const double h = dmax(dr, cut);
      if (!(dr < dmax(cut, dmax(lub_N, dmax(lub_T, lub_R))))) continue;
      const double alpha = PI * kinVisc * rad * deltat;
      double Xa, Ya, Yb1, Yc11, h_c, beta;
      if (dr < dmax(cut, lub_N)) {
        Xa = 1.0;
        h_c = dmax(dr, lub_N);
        Xa *= rad / h - rad / h_c;
        Xa *= 6.0 * alpha;
      } else
        Xa = 0.0;
      if (dr < dmax(cut, lub_T)) {
        Ya = 8.0 / 15.0;
        Yb1 = -1.0 / 5.0;
        h_c = dmax(dr, lub_T);
        beta = alpha * std::log(h_c / h);
        Ya *= 6.0 * beta;
        Yb1 *= 4.0 * beta * rad;
      } else
        Ya = Yb1 = 0.0;
      if (dr < dmax(cut, lub_R)) {
        Yc11 = 2.0 / 5.0;
        h_c = dmax(dr, lub_R);
        beta = alpha * std::log(h_c / h);
        Yc11 *= 8.0 * beta * rad * rad;
      } else
        Yc11 = 0.0;
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
      double Fx = -Xa * x12 * um_r - Ya * (umx - um_r * x12);
      double Fy = -Xa * y12 * um_r - Ya * (umy - um_r * y12);
      double Fz = -Xa * z12 * um_r - Ya * (umz - um_r * z12);
      Fx += -Yb1 * w1xrx;
      Fy += -Yb1 * w1xry;
      Fz += -Yb1 * w1xrz;
      double T1x = Yb1 * umxrx, T1y = Yb1 * umxry, T1z = Yb1 * umxrz;
      T1x += -Yc11 * (w1x - w1_r * x12);
      T1y += -Yc11 * (w1y - w1_r * y12);
      T1z += -Yc11 * (w1z - w1_r * z12);
      a.FLub.x += Fx;
      a.FLub.y += Fy;
      a.FLub.z += Fz;
      a.MLub.x += T1x;
      a.MLub.y += T1y;
      a.MLub.z += T1z;
      W.FLub.x -= Fx;
      W.FLub.y -= Fy;
      W.FLub.z -= Fz;
    }
}

// DEM::calculateObjectParticleContactForces, src/DEM.cpp:912-1138
void oracle_ctx::objectContact() {
  const double k = linearStiff, c = dampCoeff;
  const double dampCoeffTanw = 0.0;  // uninitialised local, pinned to zero
  for (Particle& a : particles)
    for (Object& o : objects) {
      const double radw = 0.5 * (a.r + o.r);
      const double x1w = a.x0.x - o.x0.x, y1w = a.x0.y - o.x0.y, z1w = a.x0.z - o.x0.z;
      const double r1w = std::sqrt(x1w * x1w + y1w * y1w + z1w * z1w);
      const double nx = x1w / r1w, ny = y1w / r1w, nz = z1w / r1w;
      const double urx = a.x1.x - o.x1.x, ury = a.x1.y - o.x1.y, urz = a.x1.z - o.x1.z;
      const double delw = (2 * radw) - r1w;
      double fnx, fny, fnz, ftx, fty, ftz;
      if (delw > 0.0) {
        const double gn = urx * nx + ury * ny + urz * nz;
        const double mu = frictionCoefPart;
        if (mu != 0.0) {
          const double ox = a.r * a.w1.x + o.r * o.w1.x;
          const double oy = a.r * a.w1.y + o.r * o.w1.y;
          const double oz = a.r * a.w1.z + o.r * o.w1.z;
          const double vx = urx + ny * oz - nz * oy - gn * nx;
          const double vy = ury + nz * ox - nx * oz - gn * ny;
          const double vz = urz + nx * oy - ny * ox - gn * nz;
          const double xi = a.xio.x * nx + a.xio.y * ny + a.xio.z * nz;
          a.xio.x -= xi * nx;
          a.xio.y -= xi * ny;
          a.xio.z -= xi * nz;
          fnx = k * delw * nx - c * gn * nx;
          fny = k * delw * ny - c * gn * ny;
          fnz = k * delw * nz - c * gn * nz;
          const double kt = 0.2 * k;
          ftx = -kt * a.xio.x;
          fty = -kt * a.xio.y;
          ftz = -kt * a.xio.z;
          const double fnn = std::sqrt(fnx * fnx + fny * fny + fnz * fnz);
          const double ftt = std::sqrt(ftx * ftx + fty * fty + ftz * ftz);
          const double fri = mu * fnn;
          const double tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
          if (fri < ftt) {
            ftx = fri * tx;
            fty = fri * ty;
            ftz = fri * tz;
            a.xio.x = -(1 / kt) * (ftx + dampCoeffTanw * vx);
            a.xio.y = -(1 / kt) * (fty + dampCoeffTanw * vy);
            a.xio.z = -(1 / kt) * (ftz + dampCoeffTanw * vz);
          } else {
            a.xio.x += vx * deltat;
            a.xio.y += vy * deltat;
            a.xio.z += vz * deltat;
          }
        } else {
          fnx = k * delw * nx - c * gn * nx;
          fny = k * delw * ny - c * gn * ny;
          fnz = k * delw * nz - c * gn * nz;
          ftx = fty = ftz = 0.0;
        }
      } else {
        fnx = fny = fnz = ftx = fty = ftz = 0.0;
        a.xio = Vec();
      }
      const double dfx = fnx + ftx, dfy = fny + fty, dfz = fnz + ftz;
      const double dtx = fty * nz - ftz * ny;
      const double dty = ftz * nx - ftx * nz;
      const double dtz = ftx * ny - fty * nx;
      a.FContact.x += dfx;
      a.FContact.y += dfy;
      a.FContact.z += dfz;
      o.FContact.x -= dfx;
      o.FContact.y -= dfy;
      o.FContact.z -= dfz;
      a.MContact.x += a.r * dtx;
      a.MContact.y += a.r * dty;
      a.MContact.z += a.r * dtz;
      o.MContact.x += o.r * dtx;
      o.MContact.y += o.r * dty;
      o.MContact.z += o.r * dtz;
    }
}

// DEM::calculateObjectParticleLubricationForces, src/DEM.cpp:1140-1340
void oracle_ctx::objectLubrication() {
  const double lub_N = lubNormal, lub_T = lubTangential, lub_R = lubRotation;
  for (Particle& a : particles)
    for (Object& o : objects) {
      const double cut = lubCutoff;
      const double rad = 0.5 * (a.r + o.r);
      double x12 = a.x0.x - o.x0.x, y12 = a.x0.y - o.x0.y, z12 = a.x0.z - o.x0.z;
      const double r12 = std::sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      const double umx = a.x1.x - o.x1.x, umy = a.x1.y - o.x1.y, umz = a.x1.z - o.x1.z;
      const double w1x = a.w1.x, w1y = a.w1.y, w1z = a.w1.z;
      const double w2x = o.w1.x, w2y = o.w1.y, w2z = o.w1.z;
      const double dr = r12 - 2.0 * rad;
      const double h = dmax(dr, cut);
      if (!(dr < dmax(cut, dmax(lub_N, dmax(lub_T, lub_R))))) continue;
      const double alpha = PI * kinVisc * rad * deltat;
      const double beta1 = o.r / a.r;
      const double beta2 = beta1 * beta1;
      const double beta3 = beta1 * beta2;
      const double beta4 = std::pow((1 + beta1), 4.0);
      double Xa, Ya, Yb1, Yb2, Yc11, Yc12, Yc21, Yc22, h_c, beta;
      if (dr < dmax(cut, lub_N)) {
        Xa = 4.0 * beta2 / beta4;
        h_c = dmax(dr, lub_N);
        Xa *= rad / h - rad / h_c;
        Xa *= 6.0 * alpha;
      } else
        Xa = 0.0;
      if (dr < dmax(cut, lub_T)) {
        Ya = 8.0 * beta1 * (2.0 + beta1 + 2.0 * beta2) / (15.0 * beta4);
        Yb1 = -4.0 * beta1 * (4.0 + beta1) / (5.0 * beta4);
        Yb2 = 4.0 * beta1 * (4.0 * beta2 + beta1) / (5.0 * beta4);
        h_c = dmax(dr, lub_T);
        beta = alpha * std::log(h_c / h);
        Ya *= 6.0 * beta;
        Yb1 *= 4.0 * beta * rad;
        Yb2 *= 4.0 * beta * rad;
      } else
        Ya = Yb1 = Yb2 = 0.0;
      if (dr < dmax(cut, lub_R)) {
        Yc11 = 16.0 * beta1 / (5.0 * beta4);
        Yc12 = 4.0 * beta2 / (5.0 * beta4);
        Yc21 = 4.0 * beta2 / (5.0 * beta4);
        Yc22 = 16.0 * beta3 / (5.0 * beta4);
        h_c = dmax(dr, lub_R);
        beta = alpha * std::log(h_c / h);
        Yc11 *= 8.0 * beta * rad * rad;
        Yc12 *= 8.0 * beta * rad * rad;
        Yc21 *= 8.0 * beta * rad * rad;
        Yc22 *= 8.0 * beta * rad * rad;
      } else
        Yc11 = Yc12 = Yc21 = Yc22 = 0.0;
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
      a.FLub.x += Fx;
      a.FLub.y += Fy;
      a.FLub.z += Fz;
      o.FLub.x -= Fx;
      o.FLub.y -= Fy;
      o.FLub.z -= Fz;
      a.MLub.x += T1x;
      a.MLub.y += T1y;
      a.MLub.z += T1z;
      o.MLub.x += T2x;
      o.MLub.y += T2y;
      o.MLub.z += T2z;
    }
}

// DEM::integration, src/DEM.cpp:2676-2765
void oracle_ctx::integration() {
  const double dt = deltat;
  for (Particle& q : particles) {
    q.x0.x += dt * q.x1.x + dt * dt * q.FTotal.x * q._m;
    q.x0.y += dt * q.x1.y + dt * dt * q.FTotal.y * q._m;
    q.x0.z += dt * q.x1.z + dt * dt * q.FTotal.z * q._m;
    q.x1.x += dt * q.FTotal.x * q._m;
    q.x1.y += dt * q.FTotal.y * q._m;
    q.x1.z += dt * q.FTotal.z * q._m;
    q.w1.x += dt * q.MTotal.x * q._I;
    q.w1.y += dt * q.MTotal.y * q._I;
    q.w1.z += dt * q.MTotal.z * q._I;
  }
  if ((int)demTimeStep >= objWaitTime)
    for (Body& b : bodies) {
      b.x0.x += dt * b.x1.x + dt * dt * b.FTotal.x * b._m;
      b.x0.y += dt * b.x1.y + dt * dt * b.FTotal.y * b._m;
      b.x0.z += dt * b.x1.z + dt * dt * b.FTotal.z * b._m;
      b.x1.x += dt * b.FTotal.x * b._m;
      b.x1.y += dt * b.FTotal.y * b._m;
      b.x1.z += dt * b.FTotal.z * b._m;
    }
  if ((int)demTimeStep >= objWaitTime)
    for (Object& o : objects) {
      o.x0.x += dt * o.x1.x + dt * dt * o.FTotal.x * o._m;
      o.x0.y += dt * o.x1.y + dt * dt * o.FTotal.y * o._m;
      o.x0.z += dt * o.x1.z + dt * dt * o.FTotal.z * o._m;
      o.x1.x += dt * o.FTotal.x * o._m;
      o.x1.y += dt * o.FTotal.y * o._m;
      o.x1.z += dt * o.FTotal.z * o._m;
      o.w1.x += dt * o.MTotal.x * o._I;
      o.w1.y += dt * o.MTotal.y * o._I;
      o.w1.z += dt * o.MTotal.z * o._I;
    }
}

// goCycle, src/main.cpp:38-67
void oracle_ctx::goCycle() {
  ++lbTime;
  if (demSolve) demStep();
  if (lbSolve && demTime >= demInitialRepeat) {
    if (demSolve) couplingStep();
    lbStep();
    if (freeSurface) fsStep();
  } else if (lbSolve && demTime <= demInitialRepeat) {
    if (demSolve) couplingStep();
  }
}

void oracle_ctx::dump(const char* path) {
  lbdump::Writer w(path);
  w.scalari("step", lbTime);
  w.scalar("demTime", demTime);
  w.scalari("demTimeStep", demTimeStep);
  if (N) {
    w.i("lbSize", {X, Y, Z});
    std::vector<uint8_t> pf(p);
    std::vector<int32_t> sol(N);
    std::vector<double> nn(N, 0.0), vx(N, 0.0), vy(N, 0.0), vz(N, 0.0), mm(N, 0.0),
        vs(N, 0.0), ff(19 * N, 0.0);
    for (size_t it = 0; it < N; ++it) {
      sol[it] = (int32_t)solid[it];
      if (hasnode[it] && isActive(it)) {
        nn[it] = n[it];
        vx[it] = ux[it];
        vy[it] = uy[it];
        vz[it] = uz[it];
        mm[it] = mass[it];
        vs[it] = visc[it];
        for (int j = 0; j < 19; ++j) ff[(size_t)j * N + it] = f[(size_t)j * N + it];
      }
    }
    w.b("type", t);
    w.b("pflag", pf);
    w.b("hasnode", hasnode);
    w.i("solid", sol);
    w.d("n", nn);
    w.d("ux", vx);
    w.d("uy", vy);
    w.d("uz", vz);
    w.d("mass", mm);
    w.d("visc", vs);
    w.d("f", ff, {19, N});
  }
  const size_t P = particles.size();
  std::vector<double> pv(3 * P);
  auto vec3 = [&](const char* name, Vec Particle::*m) {
    for (size_t i = 0; i < P; ++i) {
      const Vec v = particles[i].*m;
      pv[3 * i] = v.x;
      pv[3 * i + 1] = v.y;
      pv[3 * i + 2] = v.z;
    }
    w.d(name, pv, {P, 3});
  };
  vec3("p_x0", &Particle::x0);
  vec3("p_x1", &Particle::x1);
  vec3("p_w1", &Particle::w1);
  vec3("p_FHydro", &Particle::FHydro);
  vec3("p_MHydro", &Particle::MHydro);
  vec3("p_FContact", &Particle::FContact);
  vec3("p_MContact", &Particle::MContact);
  vec3("p_FLub", &Particle::FLub);
  vec3("p_MLub", &Particle::MLub);
  vec3("p_FRep", &Particle::FRep);
  vec3("p_FTotal", &Particle::FTotal);
  vec3("p_MTotal", &Particle::MTotal);
  vec3("p_FGrav", &Particle::FGrav);
  vec3("p_xiw", &Particle::xiw);
  vec3("p_xio", &Particle::xio);
  {
    std::vector<double> fv(P), s(9 * P);
    std::vector<int32_t> lst(50 * P);
    std::vector<double> xi(150 * P);
    for (size_t i = 0; i < P; ++i) {
      fv[i] = particles[i].fluidVolume;
      for (int k = 0; k < 9; ++k) s[9 * i + k] = particles[i].SHydro[k];
      for (int k = 0; k < 50; ++k) {
        lst[50 * i + k] = particles[i].list[k];
        xi[150 * i + k] = particles[i].xix[k];
        xi[150 * i + 50 + k] = particles[i].xiy[k];
        xi[150 * i + 100 + k] = particles[i].xiz[k];
      }
    }
    w.d("p_fluidVolume", fv);
    w.d("p_SHydro", s, {P, 9});
    w.i("p_list", lst, {P, 50});
    w.d("p_xi", xi, {P, 3, 50});
  }
  const size_t O = objects.size();
  std::vector<double> ov(3 * O);
  auto ovec = [&](const char* name, Vec Object::*m) {
    for (size_t i = 0; i < O; ++i) {
      const Vec v = objects[i].*m;
      ov[3 * i] = v.x;
      ov[3 * i + 1] = v.y;
      ov[3 * i + 2] = v.z;
    }
    w.d(name, ov, {O, 3});
  };
  ovec("o_x0", &Object::x0);
  ovec("o_x1", &Object::x1);
  ovec("o_w1", &Object::w1);
  ovec("o_FHydro", &Object::FHydro);
  ovec("o_MHydro", &Object::MHydro);
  ovec("o_FContact", &Object::FContact);
  ovec("o_MContact", &Object::MContact);
  ovec("o_FLub", &Object::FLub);
  ovec("o_MLub", &Object::MLub);
  ovec("o_FTotal", &Object::FTotal);
  const size_t W = walls.size();
  std::vector<double> wv(3 * W);
  auto wvec = [&](const char* name, Vec Wall::*m) {
    for (size_t i = 0; i < W; ++i) {
      const Vec v = walls[i].*m;
      wv[3 * i] = v.x;
      wv[3 * i + 1] = v.y;
      wv[3 * i + 2] = v.z;
    }
    w.d(name, wv, {W, 3});
  };
  wvec("w_FHydro", &Wall::FHydro);
  wvec("w_FContact", &Wall::FContact);
  wvec("w_FLub", &Wall::FLub);
  wvec("w_FTotal", &Wall::FTotal);
  const size_t B = bodies.size();
  if (B) {
    std::vector<double> bv(3 * B), bl(B);
    auto bvec = [&](const char* name, Vec Body::*m) {
      for (size_t i = 0; i < B; ++i) {
        const Vec v = bodies[i].*m;
        bv[3 * i] = v.x;
        bv[3 * i + 1] = v.y;
        bv[3 * i + 2] = v.z;
      }
      w.d(name, bv, {B, 3});
    };
    bvec("b_x0", &Body::x0);
    bvec("b_x1", &Body::x1);
    bvec("b_FSpring", &Body::FSpring);
    bvec("b_FTotal", &Body::FTotal);
    for (size_t i = 0; i < B; ++i) bl[i] = bodies[i].L;
    w.d("b_L", bl);
  }
}

// ==== C API =================================================================

extern "C" {

int oracle_create(const lbdem_config* cfg, oracle_ctx** out) {
  if (!cfg || !out) return LBDEM_ERR_INVALID;
  auto* c = new oracle_ctx();
  const int rc = c->init(cfg);
  if (rc != LBDEM_OK || !c->err.empty()) {
    *out = c;
    return rc != LBDEM_OK ? rc : LBDEM_ERR_OVERFLOW;
  }
  *out = c;
  return LBDEM_OK;
}
void oracle_destroy(oracle_ctx* c) { delete c; }
const char* oracle_last_error(const oracle_ctx* c) { return c ? c->err.c_str() : "null"; }
static int status(oracle_ctx* c) { return c->err.empty() ? LBDEM_OK : LBDEM_ERR_DEVICE_STATE; }
int oracle_dem_step(oracle_ctx* c) {
  c->demStep();
  return status(c);
}
int oracle_coupling_step(oracle_ctx* c) {
  c->couplingStep();
  return status(c);
}
int oracle_lb_step(oracle_ctx* c) {
  c->lbStep();
  return status(c);
}
int oracle_free_surface_step(oracle_ctx* c) {
  c->fsStep();
  return status(c);
}
int oracle_cycle(oracle_ctx* c, int32_t n) {
  for (int32_t k = 0; k < n && c->err.empty(); ++k) c->goCycle();
  return status(c);
}
int oracle_dump(oracle_ctx* c, const char* path) {
  c->dump(path);
  return LBDEM_OK;
}
int oracle_counters(oracle_ctx* c, int64_t* o) {
  o[0] = c->lbTime;
  o[1] = c->demTimeStep;
  o[2] = c->rebuilds;
  o[3] = (int64_t)c->activeNodes.size();
  o[4] = (int64_t)c->interfaceNodes.size();
  return LBDEM_OK;
}
double oracle_dem_time(oracle_ctx* c) { return c->demTime; }
int oracle_set_threads(int32_t n) {
  if (n < 1) return LBDEM_ERR_INVALID;
  omp_set_num_threads(n);
  return LBDEM_OK;
}
int oracle_max_threads(void) { return omp_get_max_threads(); }
int oracle_object0(oracle_ctx* c, double* o) {
  if (c->objects.empty()) return LBDEM_ERR_INVALID;
  const Object& ob = c->objects[0];
  o[0] = ob.x0.x;
  o[1] = ob.x0.y;
  o[2] = ob.x0.z;
  o[3] = ob.x1.x;
  o[4] = ob.x1.y;
  o[5] = ob.x1.z;
  return LBDEM_OK;
}

}  // extern "C"
