// Initial conditions on the device (diatom + atom) and the per-trajectory result rows.
//
//  k_ic_draws     one thread per work item: the item's random-number stream, drawn in the
//                 reference's order (RandomVector_Module.F90 RandsetVec/RanddwsVec/rand12)
//  k_sample_ic3   one thread per trajectory: SetIniCondForward (Collision_Class.F90:1065-1211)
//                 with BondLength as a 1-D Bulirsch-Stoer integration on the diatomic
//  k_results3     ApplyTransformation + Analyze/FindState of the initial and final points and
//                 the trajectories.out row (Integrator_Class.F90:701-944)
#pragma once
#include "cair_kernels.cuh"

namespace cair {

// rand12: x <- a x mod 2^64 (the reference multiplies base-256 digits), folded into a double
// by Horner from the least-significant digit with bi = 1/256.
__device__ __forceinline__ double rand12(unsigned long long& s) {
  s = s * 6364136223846793005ull;
  const double bi = 3.90625E-3;
  double r = (double)(unsigned)(s & 0xFFull);
#pragma unroll
  for (int i = 1; i < 8; ++i) r = (double)(unsigned)((s >> (8 * i)) & 0xFFull) + r * bi;
  return r * bi;
}

struct Stream {
  unsigned long long s;
  double x[100];
  __device__ void seed(long long iseed) {
    long long is = iseed;
    if (is % 2 == 0) is = is - 1;
    s = (unsigned long long)is;
    for (int i = 0; i < 100; ++i) x[i] = rand12(s);
  }
  __device__ double draw() {
    int i = (int)(99.0 * x[99]) + 1;
    double v = x[99];
    x[99] = x[i - 1];
    x[i - 1] = rand12(s);
    return v;
  }
};

constexpr int kDraws = 6;  // vibphase, rA, rB, rC, rEr, rb

#ifndef CAIR_MODEL_TU  // model-independent: built once, in the API translation unit
__global__ void k_ic_draws(int nitems, const cair_work_item* __restrict__ items,
                           const cair_level* __restrict__ levels, double* __restrict__ draws,
                           int32_t* __restrict__ item_of) {
  int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nitems) return;
  const cair_work_item W = items[it];
  const cair_level L = levels[W.ilevel];
  Stream st;
  st.seed(W.seed);
  for (int64_t k = 0; k < W.ntraj; ++k) {
    const int64_t g = W.first + k;
    st.draw();  // level pick (state-specific: the draw is made and the item's level used)
    if (L.egam != 0.0) {  // ComputeKineticEnergy rejection loop (StateInitDiatomAtom_Module.F90:299-325)
      for (int iter = 1; iter < 100000; ++iter) {
        double ra = st.draw(), rb = st.draw();
        double v1 = 2.0 * ra - 1.0, v2 = 2.0 * rb - 1.0, r = v1 * v1 + v2 * v2;
        if (r >= 1.0) continue;
        double fac = sqrt(-2.0 * log(r) / r);
        double ek = L.egam * (v1 * fac) + L.eint;
        if (ek < 0.0 || ek >= L.vmax) {
          ek = L.egam * (v2 * fac) + L.eint;
          if (ek < 0.0 || ek >= L.vmax) continue;
        }
        break;
      }
    }
    double* d = draws + kDraws * g;
    for (int j = 0; j < kDraws; ++j) d[j] = st.draw();
    item_of[g] = it;
  }
}
#endif

// BondLength (StateInitDiatomAtom_Module.F90:543-730): FuncRHS of the radial motion
struct RadialRhs {
  const DevSys& S;
  double xmui, vc_r2;
  __device__ RadialRhs(const DevSys& s, double xm, double vc) : S(s), xmui(xm), vc_r2(vc) {}
  __device__ __forceinline__ void operator()(const double (&y)[2], double (&d)[2]) const {
    double v, dv;
    diat<true>(S, y[0], v, dv);
    d[0] = y[1];
    d[1] = -xmui * (dv - 2.0 * vc_r2 / ((y[0] * y[0]) * y[0]));
  }
};

static __device__ double boltzmann_er(double ttra, double randnum) {
  const double kelvin_to_hartree = 1.0 / 3.1577513E+05;
  double betai = ttra * kelvin_to_hartree, er = 1.0;
  randnum = randnum - 1.0;
  for (int it = 0; it < 1000; ++it) {
    for (int k = 0; k < 4; ++k) er = (1.0 + er * (1.0 + er) + randnum * exp(er)) / er;
    double erri = ((1.0 + er * (1.0 + er) + randnum * exp(er)) / er) - er;
    double err = erri > 0.0 ? erri : 0.0;
    er = er + erri;
    if (err <= 1.0E-5) break;
  }
  return betai * er;
}

template <int MODEL>
__global__ void __launch_bounds__(128) k_sample_ic3(DevSys S, int64_t ntot, const cair_work_item* __restrict__ items,
                                                    const cair_level* __restrict__ levels,
                                                    const double* __restrict__ draws,
                                                    const int32_t* __restrict__ item_of, double* __restrict__ paq,
                                                    double* __restrict__ paq0, double* __restrict__ erra,
                                                    double* __restrict__ H0, double* __restrict__ bout,
                                                    int32_t* __restrict__ ipes_out, double* __restrict__ key) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ntot; g += (int64_t)gridDim.x * blockDim.x) {
    const cair_work_item W = items[item_of[g]];
    const cair_level L = levels[W.ilevel];
    const double* dr = draws + kDraws * g;
    const double* m = S.mass;
    // SetInitialState_DiatomAtom
    const double redmass_d = m[0] * m[1] / (m[0] + m[1]);
    const double xmui = 1.0 / redmass_d, xmui2 = 0.5 * xmui;
    const double jh = (double)L.jqn + 0.5;
    const double vc_r2 = xmui2 * (jh * jh);
    // BondLength from the outer turning point with zero radial velocity
    double r, rdot;
    {
      RadialRhs f(S, xmui, vc_r2);
      const double tf = dr[0] * L.tau;
      double t = 0.0, dt = tf / 10.0;
      double y[2] = {L.ro, sqrt(2.0 * xmui * 0.0)};
      double ys[2] = {L.ro * 1.0E-10, L.ro * 1.0E-10};
      double smax = 0.0, smin = 0.0;
      int irej = 0, iste = 0;
      for (int iter = 1; iter <= 10001; ++iter) {
        double rem = tf - t;
        dt = dt < rem ? dt : rem;
        bs_attempt<2, 4>(f, y, t, dt, ys, 0.5, true, smax, smin, irej, iste);
        if (fabs(t - tf) < 1.0E-08) break;
      }
      r = y[0];
      rdot = y[1];
    }
    const double omega = 2.0 * sqrt(vc_r2 * xmui2) / (r * r);
    // Compute_Coordinates_Velocities (735-833)
    const double ma = m[0], mb = m[1];
    const double fa = mb / (ma + mb), fb = -ma / (ma + mb);
    const double twopi = 3.141592653589793 * 2.0;
    const double gam = dr[1] * twopi, bet = acos(2.0 * (dr[2] - 0.5)), alp = dr[3] * twopi;
    double sb, cb, sa, ca, sg, cg;
    sincos(bet, &sb, &cb);
    sincos(alp, &sa, &ca);
    sincos(gam, &sg, &cg);
    const double u1 = cb * ca * cg - sa * sg, u2 = -(cb * ca * sg) - sa * cg;
    const double w1 = cb * sa * cg + sg * ca, w2 = -(cb * sa * sg) + ca * cg;
    const double uu1 = -(cb * sg * ca) - sa * cg;
    const double ro_ = r * omega;
    double q[3][2], qd[3][2];
    q[0][0] = fa * r * u1; q[1][0] = fa * r * u2; q[2][0] = fa * r * sb * ca;
    q[0][1] = fb * r * u1; q[1][1] = fb * r * u2; q[2][1] = fb * r * sb * ca;
    qd[0][0] = fa * (rdot * u1 + ro_ * w1); qd[1][0] = fa * (rdot * uu1 + ro_ * w2);
    qd[2][0] = fa * (rdot * (sb * ca) + ro_ * sb * sa);
    qd[0][1] = fb * (rdot * u1 + ro_ * w1); qd[1][1] = fb * (rdot * uu1 + ro_ * w2);
    qd[2][1] = fb * (rdot * (sb * ca) + ro_ * sb * sa);
    // CoordVeloc_FreeTotAngMom: Boltzmann energy and the impact parameter (Circles, one ring)
    const double er = boltzmann_er(W.ttra, dr[4]);
    double b = -W.bmax;
    if (b < 0.0) b = -sqrt(dr[5]) * b;
    // ComputeCoordinatesVelocities + ShiftCoordinates
    const double mt = m[0] + m[1], mp = m[2];
    const double redmass = mt * mp / (mt + mp);
    const double fA = -mp / (mt + mp);
    const double qx1 = fA * W.dinit;
    const double ver = sqrt(2.0 * er / redmass);
    const double ratio = b / W.dinit;
    const double verx = -ver * sqrt(1.0 - ratio * ratio), verz = -ver * ratio;
    for (int a = 0; a < 2; ++a) {
      q[0][a] = q[0][a] + qx1;
      qd[0][a] = qd[0][a] + fA * verx;
      qd[2][a] = qd[2][a] + fA * verz;
    }
    // SetPaQ: p = Tqp^T qdot over the free atoms, q = coordinates
    double y[12], dq[6];
    for (int a = 0; a < 2; ++a)
      for (int d = 0; d < 3; ++d) { y[6 + 3 * a + d] = q[d][a]; dq[3 * a + d] = qd[d][a]; }
    for (int i = 0; i < 6; ++i) y[i] = 0.0;
    for (int ip = 0; ip < 6; ++ip)
      for (int i = 0; i < 6; ++i) y[i] = y[i] + S.Tqp[ip + 9 * i] * dq[ip];
    double rpi[3];
    const double h0 = hamiltonian<MODEL>(S, S.pes[W.ipes], y, rpi);
    // SetErrorFactor: both halves from the momenta
    double ep = 0.0, eq = 0.0;
    for (int i = 0; i < 6; ++i) { ep = ep + y[i] * y[i]; eq = eq + y[i] * y[i]; }
    ep = S.eps * sqrt(ep / 6);
    eq = S.eps * sqrt(eq / 6);
    for (int i = 0; i < 12; ++i) {
      paq[12 * g + i] = y[i];
      erra[12 * g + i] = i < 6 ? ep : eq;
      paq0[12 * g + i] = i < 6 ? dq[i] : y[i];
    }
    H0[g] = h0;
    bout[g] = b;
    if (key) key[g] = ver;  // initial relative speed: slow collisions run longest
    ipes_out[g] = W.ipes;
  }
}

// Analyse the initial and final points of each trajectory and assemble its output row.
#ifndef CAIR_MODEL_TU  // model-independent: built once, in the API translation unit
__global__ void __launch_bounds__(128) k_results3(DevSys S, FsArgs F, int64_t n, const double* __restrict__ paq0,
                                                  const double* __restrict__ paq, const double* __restrict__ H0,
                                                  const double* __restrict__ H, const double* __restrict__ t,
                                                  const int32_t* __restrict__ status,
                                                  const int32_t* __restrict__ iste,
                                                  const int32_t* __restrict__ irej,
                                                  const int32_t* __restrict__ item_of,
                                                  const cair_work_item* __restrict__ items,
                                                  cair_traj_result* __restrict__ out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    double v[12];
    // ApplyTransformation: momenta -> velocities
    for (int i = 0; i < 6; ++i) {
      double a = 0.0;
      for (int j = 0; j < 6; ++j) a = a + S.Tpq[i + 9 * j] * paq[12 * k + j];
      v[i] = a;
    }
    for (int i = 6; i < 12; ++i) v[i] = paq[12 * k + i];
    cair_traj_point pi, pf;
    analyze3(S, F, paq0 + 12 * k, pi);
    analyze3(S, F, v, pf);
    cair_traj_result r;
    const int it = item_of ? item_of[k] : 0;
    r.item = it;
    r.idx = item_of ? (k - items[it].first + 1) : (k + 1);
    r.ipes = item_of ? items[it].ipes : 0;
    r.status = status[k];
    r.iste = iste[k];
    r.irej = irej[k];
    r.pad = 0;
    r.bmax = item_of ? fabs(items[it].bmax) : 0.0;
    r.b = pi.b;
    r.j_i = pi.mol[0].angmom;
    r.v_i = pi.mol[0].viba;
    r.arr_i = pi.mol[0].ipair * 16.0 + (double)pi.mol[0].itype + 0.5;
    r.j_f = pf.mol[0].angmom;
    r.v_f = pf.mol[0].viba;
    r.arr_f = pf.mol[0].ipair * 16.0 + (double)pf.mol[0].itype + 0.5;
    r.t = t[k];
    r.dH = H[k] - H0[k];
    out[k] = r;
  }
}
#endif

}  // namespace cair
