// DEM stress sums of the reference (DEM::evaluateForces, src/DEM.cpp:654-771),
// formed on the cycles whose state goes to the stress files: contactStress,
// lubStress, electroStress and hydroStress, each a 3x3 sum over the
// particles (the host divides them by the DEM volume and prints them).
//
//   contact:  -r (x) F for every particle pair (r = x_i - x_j, F = contact
//             force on i, src/DEM.cpp:1775-1783), every particle-wall contact
//             (r = the wall-normal offset, :2140-2148) and every
//             particle-impactor contact (r = x_i - x_impactor, :1127-1135)
//   electro:  -r (x) F_rep for every particle pair (:1471-1479)
//   lub:      the lubrication stresslets of both particles of every pair
//             (:2494-2512), of particles near walls (:2658-2666) and near the
//             impactor (:1325-1333), after objWaitTime
//   hydro:    the particles' hydrodynamic stresslets SHydro (:747)
//
// The pair contact and electrostatic forces are the ones the pair pass has
// stored; the wall and impactor contacts are evaluated again on copies of
// the particles' tangential springs before the gather advances them (the
// same law on the same inputs, including the fictional lid before
// objWaitTime); the stresslets are formed here in FP64 for both forms.
// With perParticle, also each particle's STotal = SHydro + SLub + SContact
// + SRep (src/DEM.cpp:748), for the particle recycle file: a pair's contact
// and electrostatic tensors go to both particles, its stresslets to each
// side.
#include "dem_forces.cuh"

namespace lbdem {

namespace {

// Stresslet coefficients of the Nguyen-Ladd lubrication of two spheres
// (Phys. Rev. E 66, 046708, 2002) in the reference's normalisation: X^G for
// the squeeze, Y^G for the shear and Y^H for the rotation terms, each scaled
// by the cut-off-limited gap functions.
struct LubStress {
  double Xg1 = 0.0, Xg2 = 0.0, Yg1 = 0.0, Yg2 = 0.0;
  double Yh11 = 0.0, Yh12 = 0.0, Yh21 = 0.0, Yh22 = 0.0;
};

// sphere a (radius ra) against sphere b (radius rb) at surface gap dr
__device__ bool lubStressSpheres(const Consts& k, double ra, double rb, double dr, LubStress& c) {
  const double cut = k.lubCut, lN = k.lubN, lT = k.lubT, lR = k.lubR;
  if (!(dr < fmax(cut, fmax(lN, fmax(lT, lR))))) return false;
  const double rad = 0.5 * (ra + rb);
  const double h = fmax(dr, cut);
  const double alpha = 3.14159265358979323846 * k.kinVisc * rad * k.dt;
  const double b1 = rb / ra, b2 = b1 * b1, b3 = b1 * b2, b5 = pow(1.0 + b1, 5.0);
  if (dr < fmax(cut, lN)) {
    const double g = (rad / h - rad / fmax(dr, lN)) * 4.0 * alpha * rad;
    c.Xg1 = 12.0 * b2 / b5 * g;
    c.Xg2 = -12.0 * b3 / b5 * g;
  }
  if (dr < fmax(cut, lT)) {
    const double g = alpha * log(fmax(dr, lT) / h) * 4.0 * rad;
    c.Yg1 = 2.0 * b1 * (4.0 - b1 + 7.0 * b2) / (5.0 * b5) * g;
    c.Yg2 = -2.0 * b2 * (4.0 * b2 - b1 + 7.0) / (5.0 * b5) * g;
  }
  if (dr < fmax(cut, lR)) {
    const double g = alpha * log(fmax(dr, lR) / h) * 8.0 * rad * rad;
    c.Yh11 = 4.0 * b1 * (2.0 - b1) / (5.0 * b5) * g;
    c.Yh12 = 2.0 * b2 * (1.0 + 7.0 * b1) / (5.0 * b5) * g;
    c.Yh21 = 2.0 * b2 * (b1 + 7.0) / (5.0 * b5) * g;
    c.Yh22 = 4.0 * b2 * (2.0 * b2 - b1) / (5.0 * b5) * g;
  }
  return true;
}

// sphere (radius ra) against a plane wall at gap dr (src/DEM.cpp:2560-2604)
__device__ bool lubStressWall(const Consts& k, double ra, double dr, LubStress& c) {
  const double cut = k.lubCut, lN = k.lubN, lT = k.lubT, lR = k.lubR;
  if (!(dr < fmax(cut, fmax(lN, fmax(lT, lR))))) return false;
  const double rad = ra, h = fmax(dr, cut);
  const double alpha = 3.14159265358979323846 * k.kinVisc * rad * k.dt;
  if (dr < fmax(cut, lN)) c.Xg1 = 1.5 * (rad / h - rad / fmax(dr, lN)) * 4.0 * alpha * rad;
  if (dr < fmax(cut, lT)) c.Yg1 = 0.7 * alpha * log(fmax(dr, lT) / h) * 4.0 * rad;
  if (dr < fmax(cut, lR)) c.Yh11 = -0.1 * alpha * log(fmax(dr, lR) / h) * 8.0 * rad * rad;
  return true;
}

// adds to S (3x3, row-major) the stresslet of one side of a lubricated pair:
//   S_ab += sgn (Xg um_r n_a n_b + Yg (n_a um_b + um_a n_b))
//           - Yh1 (n_a (w1 x n)_b + (w1 x n)_a n_b) - Yh2 (n_a (w2 x n)_b + (w2 x n)_a n_b)
// with n the unit separation of the pair and um the relative velocity
__device__ void addStresslet(double sgn, double Xg, double Yg, double Yh1, double Yh2,
                             const double* n, const double* um, const double* w1,
                             const double* w2, double* S) {
  const double umr = um[0] * n[0] + um[1] * n[1] + um[2] * n[2];
  const double a[3] = {w1[1] * n[2] - w1[2] * n[1], w1[2] * n[0] - w1[0] * n[2],
                       w1[0] * n[1] - w1[1] * n[0]};
  const double b[3] = {w2[1] * n[2] - w2[2] * n[1], w2[2] * n[0] - w2[0] * n[2],
                       w2[0] * n[1] - w2[1] * n[0]};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      S[3 * r + c] += sgn * (Xg * umr * n[r] * n[c] + Yg * (n[r] * um[c] + um[r] * n[c])) -
                      Yh1 * (n[r] * a[c] + a[r] * n[c]) - Yh2 * (n[r] * b[c] + b[r] * n[c]);
}

__device__ void addOuter(const double* r, const double* f, double* S) {
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) S[3 * a + b] -= r[a] * f[b];
}

// perParticle[c][P] += T[c] for particle p
__device__ void scatter9(double* perParticle, int P, int p, const double* T) {
  for (int c = 0; c < 9; ++c)
    if (T[c] != 0.0) atomicAdd(perParticle + (long long)c * P + p, T[c]);
}

}  // namespace

// One thread per particle; out[36] += contact, lub, electro, hydro (3x3
// row-major each). Launched between the pair pass and the gather.
__global__ void demStress(Consts k, DemArgs a, const double* SHydro, double* out,
                          double* perParticle) {
  __shared__ double acc[STRESS_N];
  for (int t = threadIdx.x; t < STRESS_N; t += blockDim.x) acc[t] = 0.0;
  __syncthreads();
  const int P = k.nPart;
  const bool afterWait = a.iscal[IS_DEMSTEP] >= k.objWaitTime;
  const int* L = a.list[a.iscal[IS_LISTCUR]];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    double C[9] = {0}, Lb[9] = {0}, E[9] = {0}, H[9];
    double Ti[9] = {0};  // this particle's share of the pair terms
    double Cown[9] = {0}, Lown[9] = {0};  // its wall and impactor terms
    double xa[3], va[3], wa[3];
    load3(a.x0, P, i, xa);
    load3(a.x1, P, i, va);
    load3(a.w1, P, i, wa);
    const double ra = a.r[i];
    for (int c = 0; c < 9; ++c) H[c] = SHydro[(long long)c * P + i];
    // pairs owned by i (the partner has the lower index)
    const int* li = L + (long long)i * MAX_N;
    for (int s = 1; s <= li[0]; ++s) {
      const int j = li[s];
      if (j >= i) continue;
      double xb[3], vb[3], wb[3];
      load3(a.x0, P, j, xb);
      const double r12v[3] = {xa[0] - xb[0], xa[1] - xb[1], xa[2] - xb[2]};
      const long long e = (long long)i * MAX_N + s;
      double fc[3], fr[3];
      for (int c = 0; c < 3; ++c) {
        fc[c] = k.mixed ? (double)((const float*)a.pairbuf)[e * PAIR_VALS + c]
                        : a.pairbuf[e * PAIR_VALS + c];
        fr[c] = k.mixed ? (double)((const float*)a.pairbuf)[e * PAIR_VALS + 15 + c]
                        : a.pairbuf[e * PAIR_VALS + 15 + c];
      }
      double T[9] = {0};  // contact + electrostatic of the pair, for both particles
      addOuter(r12v, fc, C);
      addOuter(r12v, fr, E);
      if (perParticle) {
        addOuter(r12v, fc, T);
        addOuter(r12v, fr, T);
        for (int c = 0; c < 9; ++c) Ti[c] += T[c];
      }
      double S2[9] = {0};
      if (afterWait) {
        const double rb = a.r[j];
        const double r12 = sqrt(r12v[0] * r12v[0] + r12v[1] * r12v[1] + r12v[2] * r12v[2]);
        LubStress ls;
        if (lubStressSpheres(k, ra, rb, r12 - (ra + rb), ls)) {
          load3(a.x1, P, j, vb);
          load3(a.w1, P, j, wb);
          const double n[3] = {r12v[0] / r12, r12v[1] / r12, r12v[2] / r12};
          const double um[3] = {va[0] - vb[0], va[1] - vb[1], va[2] - vb[2]};
          double S1[9] = {0};
          addStresslet(1.0, ls.Xg1, ls.Yg1, ls.Yh11, ls.Yh12, n, um, wa, wb, S1);
          addStresslet(-1.0, ls.Xg2, ls.Yg2, ls.Yh21, ls.Yh22, n, um, wa, wb, S2);
          for (int c = 0; c < 9; ++c) {
            Lb[c] += S1[c] + S2[c];
            Ti[c] += S1[c];
          }
        }
      }
      if (perParticle) {
        for (int c = 0; c < 9; ++c) T[c] += S2[c];
        scatter9(perParticle, P, j, T);
      }
    }
    double xiw[3], xio[3], df[3], dt[3];
    load3(a.xiw, P, i, xiw);
    load3(a.xio, P, i, xio);
    const double zero3[3] = {0.0, 0.0, 0.0};
    if (afterWait) {
      for (int w = 0; w < k.nWall; ++w) {
        const DeviceWall& W = a.walls[w];
        double o[3];
        for (int c = 0; c < 3; ++c) o[c] = (xa[c] - W.p[c]) * W.n[c] * W.n[c];
        const double r12 = sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        LubStress ls;
        if (!lubStressWall(k, ra, r12 - ra, ls)) continue;
        const double n[3] = {o[0] / r12, o[1] / r12, o[2] / r12};
        addStresslet(1.0, ls.Xg1, ls.Yg1, ls.Yh11, 0.0, n, va, wa, zero3, Lown);
      }
      for (int ob = 0; ob < k.nObj; ++ob) {
        const double* B = a.obj + ob * OB_STRIDE;
        const PairGeom<double> g = pairGeomD(0.5 * (ra + B[OB_R]), xa, B + OB_X0, va, B + OB_X1);
        objContactOne(k, ra, B[OB_R], g, wa, B + OB_W1, xio, df, dt);
        const double r[3] = {xa[0] - B[OB_X0], xa[1] - B[OB_X0 + 1], xa[2] - B[OB_X0 + 2]};
        addOuter(r, df, Cown);
      }
      for (int ob = 0; ob < k.nObj; ++ob) {
        const double* B = a.obj + ob * OB_STRIDE;
        const double r[3] = {xa[0] - B[OB_X0], xa[1] - B[OB_X0 + 1], xa[2] - B[OB_X0 + 2]};
        const double r12 = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        LubStress ls;
        if (!lubStressSpheres(k, ra, B[OB_R], r12 - (ra + B[OB_R]), ls)) continue;
        const double n[3] = {r[0] / r12, r[1] / r12, r[2] / r12};
        const double um[3] = {va[0] - B[OB_X1], va[1] - B[OB_X1 + 1], va[2] - B[OB_X1 + 2]};
        addStresslet(1.0, ls.Xg1, ls.Yg1, ls.Yh11, ls.Yh12, n, um, wa, B + OB_W1, Lown);
      }
    } else {
      // the fictional lid advances the wall spring before the walls do
      double nst[3] = {0.0, 0.0, 0.0};
      const double ylid = xa[1] - (k.demSize[1] - 0.3);
      wallContactOne(k, ra, va, wa, xiw, 0.0, ylid, 0.0, sqrt(ylid * ylid), nst, df, dt);
    }
    {
      double nst[3] = {0.0, 0.0, 0.0};
      for (int w = 0; w < k.nWall; ++w) {
        const DeviceWall& W = a.walls[w];
        double o[3];
        for (int c = 0; c < 3; ++c) o[c] = (xa[c] - W.p[c]) * W.n[c] * W.n[c];
        const double r1w = sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        wallContactOne(k, ra, va, wa, xiw, o[0], o[1], o[2], r1w, nst, df, dt);
        addOuter(o, df, Cown);
      }
    }
    if (perParticle) {
      // pair terms (Ti), then its own walls, impactor and hydrodynamics
      double T[9];
      for (int c = 0; c < 9; ++c) T[c] = Ti[c] + (Cown[c] + Lown[c]) + H[c];
      scatter9(perParticle, P, i, T);
    }
    for (int c = 0; c < 9; ++c) {
      C[c] += Cown[c];
      Lb[c] += Lown[c];
      if (C[c] != 0.0) atomicAdd(&acc[c], C[c]);
      if (Lb[c] != 0.0) atomicAdd(&acc[9 + c], Lb[c]);
      if (E[c] != 0.0) atomicAdd(&acc[18 + c], E[c]);
      if (H[c] != 0.0) atomicAdd(&acc[27 + c], H[c]);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < STRESS_N; t += blockDim.x)
    if (acc[t] != 0.0) atomicAdd(out + t, acc[t]);
}

}  // namespace lbdem
