// DEM force laws, templated on the arithmetic type: double for the plain
// form (every expression as the reference evaluates it) and float for the
// mixed form, whose callers compute the pair geometry (gap and normal) in
// double for near-contact pairs and round it.
//
// Each law takes the geometry its caller computed: the centre distance r12,
// the gap r12 - 2 rad (r1w - r for walls) and the unit normal, so that one
// geometry serves the contact, lubrication and repulsion laws of a pair.
//
// Reference: DEM::calculateParticleContactForces (src/DEM.cpp:1506-1700),
// lubrication of pairs (:2325-2491) and of particle and impactor
// (:1158-1323), calculateParticleElectroForces (:1413-1449), particle-wall
// contact (:1956-2108) and lid (:2166-2292), particle-wall lubrication
// (:2541-2670), particle-impactor contact (:921-1090).
#pragma once
#include "kernels_decl.h"

namespace lbdem {

__device__ __forceinline__ double tsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float tsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double texp(double x) { return exp(x); }
__device__ __forceinline__ float texp(float x) { return expf(x); }
__device__ __forceinline__ double tlog(double x) { return log(x); }
__device__ __forceinline__ float tlog(float x) { return logf(x); }
__device__ __forceinline__ double tpow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float tpow(float x, float y) { return powf(x, y); }
template <typename T>
__device__ __forceinline__ T tmax(T a, T b) {
  return a > b ? a : b;
}

// Geometry of a sphere pair (a, b): centre distance, gap r12 - 2 rad with
// rad the mean radius, unit normal from b to a, relative velocity va - vb.
template <typename T>
struct PairGeom {
  T r12, gap, n[3], u[3];
};

// The plain form's geometry, as each force law of the reference computes it.
__device__ __forceinline__ PairGeom<double> pairGeomD(double rad, const double* xa,
                                                      const double* xb, const double* va,
                                                      const double* vb) {
  PairGeom<double> g;
  const double x12 = xa[0] - xb[0], y12 = xa[1] - xb[1], z12 = xa[2] - xb[2];
  g.r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
  g.gap = g.r12 - 2.0 * rad;
  g.n[0] = x12 / g.r12;
  g.n[1] = y12 / g.r12;
  g.n[2] = z12 / g.r12;
  g.u[0] = va[0] - vb[0];
  g.u[1] = va[1] - vb[1];
  g.u[2] = va[2] - vb[2];
  return g;
}

// Pair contact: linear spring-dashpot normal force, tangential spring xi
// (in/out) with Coulomb limit. out: force on a (3), tangential torque arm
// n x ft scaled later by the radius (3).
template <typename T>
__device__ void pairContact(const Consts& k, T ra, T rb, const PairGeom<T>& g, const T* wa,
                            const T* wb, T* xi, T* out) {
  const T nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const T urx = g.u[0], ury = g.u[1], urz = g.u[2];
  const T gn = urx * nx + ury * ny + urz * nz;
  const T mu = T(k.mu), kk = T(k.k), c = T(k.c);
  const T del = -g.gap;  // 2 rad - r12
  T fnx, fny, fnz, ftx, fty, ftz;
  if (del > T(0)) {
    if (mu != T(0)) {
      const T ox = ra * wa[0] + rb * wb[0];
      const T oy = ra * wa[1] + rb * wb[1];
      const T oz = ra * wa[2] + rb * wb[2];
      const T vx = urx + ny * oz - nz * oy - gn * nx;
      const T vy = ury + nz * ox - nx * oz - gn * ny;
      const T vz = urz + nx * oy - ny * ox - gn * nz;
      const T xi12 = xi[0] * nx + xi[1] * ny + xi[2] * nz;
      xi[0] -= xi12 * nx;
      xi[1] -= xi12 * ny;
      xi[2] -= xi12 * nz;
      fnx = kk * del * nx - c * gn * nx;
      fny = kk * del * ny - c * gn * ny;
      fnz = kk * del * nz - c * gn * nz;
      const T kt = T(0.2) * kk;
      const T dct = k.kinVisc == 0.0 ? c : T(0);
      ftx = -kt * xi[0] - dct * vx;
      fty = -kt * xi[1] - dct * vy;
      ftz = -kt * xi[2] - dct * vz;
      const T fnn = tsqrt(fnx * fnx + fny * fny + fnz * fnz);
      const T ftt = tsqrt(ftx * ftx + fty * fty + ftz * ftz);
      const T fri = mu * fnn;
      const T tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
      const T dtt = T(k.dt);
      xi[0] += vx * dtt;
      xi[1] += vy * dtt;
      xi[2] += vz * dtt;
      if (fri < ftt) {
        ftx = fri * tx;
        fty = fri * ty;
        ftz = fri * tz;
        xi[0] = -(T(1) / kt) * (ftx + dct * vx);
        xi[1] = -(T(1) / kt) * (fty + dct * vy);
        xi[2] = -(T(1) / kt) * (ftz + dct * vz);
      }
    } else {
      fnx = kk * del * nx - c * gn * nx;
      fny = kk * del * ny - c * gn * ny;
      fnz = kk * del * nz - c * gn * nz;
      ftx = fty = ftz = T(0);
    }
  } else {
    fnx = fny = fnz = ftx = fty = ftz = T(0);
    xi[0] = xi[1] = xi[2] = T(0);
  }
  out[0] = fnx + ftx;
  out[1] = fny + fty;
  out[2] = fnz + ftz;
  out[3] = fty * nz - ftz * ny;
  out[4] = ftz * nx - ftx * nz;
  out[5] = ftx * ny - fty * nx;
}

// Nguyen-Ladd lubrication of a sphere pair, or of a particle (a) and an
// impactor (b). Returns false outside the cut-off; out: force on a (3),
// torque on a (3), torque on b (3).
template <typename T>
__device__ bool pairLub(const Consts& k, T ra, T rb, const PairGeom<T>& g, const T* wa,
                        const T* wb, T* out) {
  const T lub_N = T(k.lubN), lub_T = T(k.lubT), lub_R = T(k.lubR), cut = T(k.lubCut);
  const T rad = T(0.5) * (ra + rb);
  const T umx = g.u[0], umy = g.u[1], umz = g.u[2];
  const T w1x = wa[0], w1y = wa[1], w1z = wa[2];
  const T w2x = wb[0], w2y = wb[1], w2z = wb[2];
  const T dr = g.gap;
  const T h = tmax(dr, cut);
  if (!(dr < tmax(cut, tmax(lub_N, tmax(lub_T, lub_R))))) return false;
  const T alpha = T(3.14159265358979323846) * T(k.kinVisc) * rad * T(k.dt);
  const T beta1 = rb / ra;
  const T beta2 = beta1 * beta1;
  const T beta3 = beta1 * beta2;
  const T beta4 = tpow((T(1) + beta1), T(4));
  T Xa, Ya, Yb1, Yb2, Yc11, Yc12, Yc21, Yc22, h_c, beta;
  if (dr < tmax(cut, lub_N)) {
    Xa = T(4) * beta2 / beta4;
    h_c = tmax(dr, lub_N);
    Xa *= rad / h - rad / h_c;
    Xa *= T(6) * alpha;
  } else {
    Xa = T(0);
  }
  if (dr < tmax(cut, lub_T)) {
    Ya = T(8) * beta1 * (T(2) + beta1 + T(2) * beta2) / (T(15) * beta4);
    Yb1 = -T(4) * beta1 * (T(4) + beta1) / (T(5) * beta4);
    Yb2 = T(4) * beta1 * (T(4) * beta2 + beta1) / (T(5) * beta4);
    h_c = tmax(dr, lub_T);
    beta = alpha * tlog(h_c / h);
    Ya *= T(6) * beta;
    Yb1 *= T(4) * beta * rad;
    Yb2 *= T(4) * beta * rad;
  } else {
    Ya = Yb1 = Yb2 = T(0);
  }
  if (dr < tmax(cut, lub_R)) {
    Yc11 = T(16) * beta1 / (T(5) * beta4);
    Yc12 = T(4) * beta2 / (T(5) * beta4);
    Yc21 = T(4) * beta2 / (T(5) * beta4);
    Yc22 = T(16) * beta3 / (T(5) * beta4);
    h_c = tmax(dr, lub_R);
    beta = alpha * tlog(h_c / h);
    Yc11 *= T(8) * beta * rad * rad;
    Yc12 *= T(8) * beta * rad * rad;
    Yc21 *= T(8) * beta * rad * rad;
    Yc22 *= T(8) * beta * rad * rad;
  } else {
    Yc11 = Yc12 = Yc21 = Yc22 = T(0);
  }
  const T x12 = g.n[0], y12 = g.n[1], z12 = g.n[2];
  const T um_r = umx * x12 + umy * y12 + umz * z12;
  const T w1_r = w1x * x12 + w1y * y12 + w1z * z12;
  const T w2_r = w2x * x12 + w2y * y12 + w2z * z12;
  const T umxrx = umy * z12 - umz * y12;
  const T umxry = umz * x12 - umx * z12;
  const T umxrz = umx * y12 - umy * x12;
  const T w1xrx = w1y * z12 - w1z * y12;
  const T w1xry = w1z * x12 - w1x * z12;
  const T w1xrz = w1x * y12 - w1y * x12;
  const T w2xrx = w2y * z12 - w2z * y12;
  const T w2xry = w2z * x12 - w2x * z12;
  const T w2xrz = w2x * y12 - w2y * x12;
  T Fx = -Xa * um_r * x12 - Ya * (umx - um_r * x12);
  T Fy = -Xa * um_r * y12 - Ya * (umy - um_r * y12);
  T Fz = -Xa * um_r * z12 - Ya * (umz - um_r * z12);
  Fx += -Yb1 * w1xrx + Yb2 * w2xrx;
  Fy += -Yb1 * w1xry + Yb2 * w2xry;
  Fz += -Yb1 * w1xrz + Yb2 * w2xrz;
  T T1x = Yb1 * umxrx, T1y = Yb1 * umxry, T1z = Yb1 * umxrz;
  T T2x = -Yb2 * umxrx, T2y = -Yb2 * umxry, T2z = -Yb2 * umxrz;
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

// Exponential electrostatic repulsion of a pair; out: force on a.
template <typename T>
__device__ void pairRep(const Consts& k, const PairGeom<T>& g, T* out) {
  const T nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const T del = -g.gap;
  const T el = T(k.electro);
  if (del <= T(0)) {
    const T e = texp(del / T(k.debye));
    out[0] = el * e * nx;
    out[1] = el * e * ny;
    out[2] = el * e * nz;
  } else {
    out[0] = el * nx;
    out[1] = el * ny;
    out[2] = el * nz;
  }
}

// Particle-wall contact or the lid: (x1w, y1w, z1w) the particle's offset
// from the wall along its normal, r1w its length; nstale the normal kept
// from the last wall in contact (in/out); xiw the wall spring (in/out).
template <typename T>
__device__ void wallContactOne(const Consts& k, T r, const T* v, const T* w, T* xiw, T x1w,
                               T y1w, T z1w, T r1w, T* nstale, T* df, T* dt) {
  const T delw = r - r1w;
  T fnx, fny, fnz, ftx, fty, ftz;
  if (delw > T(0)) {
    nstale[0] = x1w / r1w;
    nstale[1] = y1w / r1w;
    nstale[2] = z1w / r1w;
    const T nx = nstale[0], ny = nstale[1], nz = nstale[2];
    const T urx = v[0], ury = v[1], urz = v[2];
    const T gn = urx * nx + ury * ny + urz * nz;
    const T kk = T(k.k), c = T(k.c);
    if (k.mu != 0.0) {
      const T ox = r * w[0], oy = r * w[1], oz = r * w[2];
      const T vx = urx + ny * oz - nz * oy - gn * nx;
      const T vy = ury + nz * ox - nx * oz - gn * ny;
      const T vz = urz + nx * oy - ny * ox - gn * nz;
      const T xi = xiw[0] * nx + xiw[1] * ny + xiw[2] * nz;
      xiw[0] -= xi * nx;
      xiw[1] -= xi * ny;
      xiw[2] -= xi * nz;
      fnx = kk * delw * nx - c * gn * nx;
      fny = kk * delw * ny - c * gn * ny;
      fnz = kk * delw * nz - c * gn * nz;
      const T kt = T(0.2) * kk;
      const T dct = k.kinVisc == 0.0 ? c : T(0);
      ftx = -kt * xiw[0] - dct * vx;
      fty = -kt * xiw[1] - dct * vy;
      ftz = -kt * xiw[2] - dct * vz;
      const T fnn = tsqrt(fnx * fnx + fny * fny + fnz * fnz);
      const T ftt = tsqrt(ftx * ftx + fty * fty + ftz * ftz);
      const T fri = T(k.mu) * fnn;
      const T tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
      const T dtt = T(k.dt);
      xiw[0] += vx * dtt;
      xiw[1] += vy * dtt;
      xiw[2] += vz * dtt;
      if (fri < ftt) {
        ftx = fri * tx;
        fty = fri * ty;
        ftz = fri * tz;
        xiw[0] = -(T(1) / kt) * (ftx + dct * vx);
        xiw[1] = -(T(1) / kt) * (fty + dct * vy);
        xiw[2] = -(T(1) / kt) * (ftz + dct * vz);
      }
    } else {
      fnx = kk * delw * nx - c * gn * nx;
      fny = kk * delw * ny - c * gn * ny;
      fnz = kk * delw * nz - c * gn * nz;
      ftx = fty = ftz = T(0);
    }
  } else {
    fnx = fny = fnz = ftx = fty = ftz = T(0);
    xiw[0] = xiw[1] = xiw[2] = T(0);
  }
  df[0] = fnx + ftx;
  df[1] = fny + fty;
  df[2] = fnz + ftz;
  dt[0] = fty * nstale[2] - ftz * nstale[1];
  dt[1] = ftz * nstale[0] - ftx * nstale[2];
  dt[2] = ftx * nstale[1] - fty * nstale[0];
}

// Particle-wall lubrication: (x12, y12, z12) the offset from the wall, r12
// its length. Returns false outside the cut-off.
template <typename T>
__device__ bool wallLubOne(const Consts& k, T rad, const T* v, const T* w, T x12, T y12, T z12,
                           T r12, T* F, T* Tq) {
  const T cut = T(k.lubCut), lub_N = T(k.lubN), lub_T = T(k.lubT), lub_R = T(k.lubR);
  const T umx = v[0], umy = v[1], umz = v[2];
  const T w1x = w[0], w1y = w[1], w1z = w[2];
  const T dr = r12 - rad;
  const T h = tmax(dr, cut);
  if (!(dr < tmax(cut, tmax(lub_N, tmax(lub_T, lub_R))))) return false;
  const T alpha = T(3.14159265358979323846) * T(k.kinVisc) * rad * T(k.dt);
  T Xa, Ya, Yb1, Yc11, h_c, beta;
  if (dr < tmax(cut, lub_N)) {
    Xa = T(1);
    h_c = tmax(dr, lub_N);
    Xa *= rad / h - rad / h_c;
    Xa *= T(6) * alpha;
  } else {
    Xa = T(0);
  }
  if (dr < tmax(cut, lub_T)) {
    Ya = T(8.0 / 15.0);
    Yb1 = T(-1.0 / 5.0);
    h_c = tmax(dr, lub_T);
    beta = alpha * tlog(h_c / h);
    Ya *= T(6) * beta;
    Yb1 *= T(4) * beta * rad;
  } else {
    Ya = Yb1 = T(0);
  }
  if (dr < tmax(cut, lub_R)) {
    Yc11 = T(2.0 / 5.0);
    h_c = tmax(dr, lub_R);
    beta = alpha * tlog(h_c / h);
    Yc11 *= T(8) * beta * rad * rad;
  } else {
    Yc11 = T(0);
  }
  x12 /= r12;
  y12 /= r12;
  z12 /= r12;
  const T um_r = umx * x12 + umy * y12 + umz * z12;
  const T w1_r = w1x * x12 + w1y * y12 + w1z * z12;
  const T umxrx = umy * z12 - umz * y12;
  const T umxry = umz * x12 - umx * z12;
  const T umxrz = umx * y12 - umy * x12;
  const T w1xrx = w1y * z12 - w1z * y12;
  const T w1xry = w1z * x12 - w1x * z12;
  const T w1xrz = w1x * y12 - w1y * x12;
  F[0] = -Xa * x12 * um_r - Ya * (umx - um_r * x12);
  F[1] = -Xa * y12 * um_r - Ya * (umy - um_r * y12);
  F[2] = -Xa * z12 * um_r - Ya * (umz - um_r * z12);
  F[0] += -Yb1 * w1xrx;
  F[1] += -Yb1 * w1xry;
  F[2] += -Yb1 * w1xrz;
  Tq[0] = Yb1 * umxrx;
  Tq[1] = Yb1 * umxry;
  Tq[2] = Yb1 * umxrz;
  Tq[0] += -Yc11 * (w1x - w1_r * x12);
  Tq[1] += -Yc11 * (w1y - w1_r * y12);
  Tq[2] += -Yc11 * (w1z - w1_r * z12);
  return true;
}

// Particle-impactor contact; dampCoeffTanw is an uninitialised local in the
// reference, zero under the pinned build.
template <typename T>
__device__ void objContactOne(const Consts& k, T ra, T ro, const PairGeom<T>& g, const T* wa,
                              const T* wo, T* xio, T* df, T* dt) {
  const T nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const T urx = g.u[0], ury = g.u[1], urz = g.u[2];
  const T delw = -g.gap;  // 2 radw - r1w
  const T dampCoeffTanw = T(0);
  const T kk = T(k.k), c = T(k.c);
  T fnx, fny, fnz, ftx, fty, ftz;
  if (delw > T(0)) {
    const T gn = urx * nx + ury * ny + urz * nz;
    if (k.mu != 0.0) {
      const T ox = ra * wa[0] + ro * wo[0];
      const T oy = ra * wa[1] + ro * wo[1];
      const T oz = ra * wa[2] + ro * wo[2];
      const T vx = urx + ny * oz - nz * oy - gn * nx;
      const T vy = ury + nz * ox - nx * oz - gn * ny;
      const T vz = urz + nx * oy - ny * ox - gn * nz;
      const T xi = xio[0] * nx + xio[1] * ny + xio[2] * nz;
      xio[0] -= xi * nx;
      xio[1] -= xi * ny;
      xio[2] -= xi * nz;
      fnx = kk * delw * nx - c * gn * nx;
      fny = kk * delw * ny - c * gn * ny;
      fnz = kk * delw * nz - c * gn * nz;
      const T kt = T(0.2) * kk;
      ftx = -kt * xio[0];
      fty = -kt * xio[1];
      ftz = -kt * xio[2];
      const T fnn = tsqrt(fnx * fnx + fny * fny + fnz * fnz);
      const T ftt = tsqrt(ftx * ftx + fty * fty + ftz * ftz);
      const T fri = T(k.mu) * fnn;
      const T tx = ftx / ftt, ty = fty / ftt, tz = ftz / ftt;
      if (fri < ftt) {
        ftx = fri * tx;
        fty = fri * ty;
        ftz = fri * tz;
        xio[0] = -(T(1) / kt) * (ftx + dampCoeffTanw * vx);
        xio[1] = -(T(1) / kt) * (fty + dampCoeffTanw * vy);
        xio[2] = -(T(1) / kt) * (ftz + dampCoeffTanw * vz);
      } else {
        const T dtt = T(k.dt);
        xio[0] += vx * dtt;
        xio[1] += vy * dtt;
        xio[2] += vz * dtt;
      }
    } else {
      fnx = kk * delw * nx - c * gn * nx;
      fny = kk * delw * ny - c * gn * ny;
      fnz = kk * delw * nz - c * gn * nz;
      ftx = fty = ftz = T(0);
    }
  } else {
    fnx = fny = fnz = ftx = fty = ftz = T(0);
    xio[0] = xio[1] = xio[2] = T(0);
  }
  df[0] = fnx + ftx;
  df[1] = fny + fty;
  df[2] = fnz + ftz;
  dt[0] = fty * nz - ftz * ny;
  dt[1] = ftz * nx - ftx * nz;
  dt[2] = ftx * ny - fty * nx;
}

__device__ __forceinline__ void load3(const double* a, int P, int i, double* v) {
  v[0] = a[i];
  v[1] = a[P + i];
  v[2] = a[2 * P + i];
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
// 2742-2760), by the last block of the gather once every block's impactor
// and wall sums are in. The record is read with ld.global.cg (past L1, so
// no line this block cached earlier in the kernel can be stale) in one batch
// of independent loads, then written back.
// The bodies' part of a DEM step, by one thread in the reference's loop
// order: the resets of evaluateForces (src/DEM.cpp:688-713), from objWaitTime
// on the springs of DEM::bodyObjectInteraction (:798-869, into the objects'
// FSpring, before their totals), the bodies' totals (:792-794) and from
// objWaitTime on their integration (:2730-2739).
static __device__ __noinline__ void demBodies(const Consts& k, const DemArgs& a, int stepNo) {
  for (int o = 0; o < k.nObj; ++o)
    for (int c = 0; c < 3; ++c) a.obj[o * OB_STRIDE + OB_FSPRING + c] = 0.0;
  for (int b = 0; b < k.nBody; ++b)
    for (int c = 0; c < 3; ++c) a.body[b * BD_STRIDE + BD_FSPRING + c] = 0.0;
  if (stepNo >= k.objWaitTime)
    for (int b = 0; b < k.nBody; ++b) {
      double* bd = a.body + b * BD_STRIDE;
      for (int o = 0; o < k.nObj; ++o) {
        double* ob = a.obj + o * OB_STRIDE;
        double fs = 0.0, fdo = 0.0, fdb = 0.0;
        bd[BD_L] = bd[BD_X0 + 1] - ob[OB_X0 + 1];
        const double rx = bd[BD_X0] - ob[OB_X0], ry = bd[BD_X0 + 1] - ob[OB_X0 + 1],
                     rz = bd[BD_X0 + 2] - ob[OB_X0 + 2];
        const double rn = sqrt(rx * rx + ry * ry + rz * rz);
        const double ny = ry / rn;
        const double del = bd[BD_L0] - bd[BD_L];
        const double kb = bd[BD_K];
        const double bodyDamp = 2.0 * sqrt(bd[BD_M] * kb) * k.springDamp;
        const double objDamp = 2.0 * sqrt(ob[OB_MASS] * kb) * k.springDamp;
        const double sigma = bd[BD_R];
        if (k.nonLinType == 0) {  // spring
          fs = kb * del * ny;
        } else if (k.nonLinType >= 1 && k.nonLinType <= 4) {
          if (k.nonLinType == 1) {  // spring-dashpot
            fs = (kb * del) * ny;
          } else if (k.nonLinType == 2) {  // spring-dashpot-cubic
            fs = (kb * del + k.k13 * kb * (del * del * del)) * ny;
          } else if (k.nonLinType == 3) {  // spring-dashpot-repLJ
            fs = (kb * del + (24.0 * k.epsilon / rn) * 2.0 * pow(sigma / rn, 12.0)) * ny;
          } else {  // spring-dashpot-WCA
            const double wcacut = pow(2.0, 1.0 / 6.0) * sigma;
            if (rn <= wcacut)
              fs = (kb * del + (24.0 * k.epsilon / rn) *
                                   (2.0 * pow(sigma / rn, 12.0) - pow(sigma / rn, 6.0))) *
                   ny;
            else
              fs = (kb * del) * ny;
          }
          fdo = -ob[OB_X1 + 1] * objDamp;
          fdb = -bd[BD_X1 + 1] * bodyDamp;
        }
        ob[OB_FSPRING + 1] -= fs;
        bd[BD_FSPRING + 1] += fs;
        ob[OB_FSPRING + 1] += fdo;
        bd[BD_FSPRING + 1] += fdb;
      }
    }
  const double dtt = k.dt;
  for (int b = 0; b < k.nBody; ++b) {
    double* bd = a.body + b * BD_STRIDE;
    double FT[3];
    for (int c = 0; c < 3; ++c) {
      FT[c] = 0.0 + (bd[BD_FGRAV + c] + bd[BD_FSPRING + c]);
      bd[BD_FTOTAL + c] = FT[c];
    }
    if (stepNo >= k.objWaitTime) {
      const double invm = bd[BD_INVM];
      for (int c = 0; c < 3; ++c) {
        bd[BD_X0 + c] = bd[BD_X0 + c] + (dtt * bd[BD_X1 + c] + dtt * dtt * FT[c] * invm);
        bd[BD_X1 + c] = bd[BD_X1 + c] + dtt * FT[c] * invm;
      }
    }
  }
}

__device__ __forceinline__ void demObjectsTail(const Consts& k, const DemArgs& a) {
  const int stepNo = a.iscal[IS_DEMSTEP];
  if (k.nBody > 0) {  // uniform over the block
    if (threadIdx.x == 0) demBodies(k, a, stepNo);
    __syncthreads();
  }
  const int o = threadIdx.x;
  if (o < k.nObj) {
    double* ob = a.obj + o * OB_STRIDE;
    double FH[3], FC[3], FL[3], FG[3], FS[3], MH[3], MC[3], ML[3], X0[3], X1[3], W1[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      FH[c] = __ldcg(ob + OB_FHYDRO + c);
      FC[c] = __ldcg(ob + OB_FCONTACT + c);
      FL[c] = __ldcg(ob + OB_FLUB + c);
      FG[c] = __ldcg(ob + OB_FGRAV + c);
      FS[c] = k.nBody > 0 ? __ldcg(ob + OB_FSPRING + c) : 0.0;
      MH[c] = __ldcg(ob + OB_MHYDRO + c);
      MC[c] = __ldcg(ob + OB_MCONTACT + c);
      ML[c] = __ldcg(ob + OB_MLUB + c);
      X0[c] = __ldcg(ob + OB_X0 + c);
      X1[c] = __ldcg(ob + OB_X1 + c);
      W1[c] = __ldcg(ob + OB_W1 + c);
    }
    const double invm = __ldcg(ob + OB_INVM), invI = __ldcg(ob + OB_INVI);
    const double dtt = k.dt;
    double FT[3], MT[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      FT[c] = 0.0 + ((((FH[c] + FC[c]) + FL[c]) + FG[c]) + FS[c]);
      MT[c] = 0.0 + ((MH[c] + MC[c]) + ML[c]);
      ob[OB_FTOTAL + c] = FT[c];
      ob[OB_MTOTAL + c] = MT[c];
    }
    if (stepNo >= k.objWaitTime)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ob[OB_X0 + c] = X0[c] + (dtt * X1[c] + dtt * dtt * FT[c] * invm);
        ob[OB_X1 + c] = X1[c] + dtt * FT[c] * invm;
        ob[OB_W1 + c] = W1[c] + dtt * MT[c] * invI;
      }
  }
  if (o < k.nWall) {
    double* w = a.wallF + o * 12;
    double v[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) v[c] = __ldcg(w + c);
#pragma unroll
    for (int c = 0; c < 3; ++c) w[9 + c] = 0.0 + (((v[c] + v[3 + c]) + v[6 + c]) + 0.0);
  }
}

}  // namespace lbdem
