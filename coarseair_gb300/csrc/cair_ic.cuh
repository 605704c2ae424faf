// Initial conditions on the device (diatom + atom, diatom + diatom) and the per-trajectory result rows.
//
//  k_ic_draws     one thread per random-number stream (a work item and the impact-parameter rings
//                 that continue it), drawn in the reference's order (RandomVector_Module.F90
//                 RandsetVec/RanddwsVec/rand12)
//  k_sample_ic3/4 one thread per trajectory: SetIniCondForward (Collision_Class.F90:1065-1211)
//                 for diatom + atom / diatom + diatom, BondLength as a 1-D Bulirsch-Stoer
//                 integration on the diatomic
//  k_results      ApplyTransformation + Analyze/FindState of the initial and final points and
//                 the trajectories.out row (Integrator_Class.F90:701-944)
#pragma once
#include "cair_kernels.cuh"

namespace cair {

// rand12: x <- a x mod 2^64 (the reference multiplies base-256 digits), folded into a double
// by Horner from the least-significant digit with bi = 1/256.
__host__ __device__ __forceinline__ double rand12(unsigned long long& s) {
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
  __host__ __device__ void seed(long long iseed) {
    long long is = iseed;
    if (is % 2 == 0) is = is - 1;
    s = (unsigned long long)is;
    for (int i = 0; i < 100; ++i) x[i] = rand12(s);
  }
  __host__ __device__ double draw() {
    int i = (int)(99.0 * x[99]) + 1;
    double v = x[99];
    x[99] = x[i - 1];
    x[i - 1] = rand12(s);
    return v;
  }
};

// Draws kept per trajectory: per diatom (vibphase, rA, rB, rC), then rEr and rb
constexpr int kDraws = 10;

// True when work item it continues the random-number stream of item it - 1: the next impact-parameter
// ring of the same stream (same seed, skip = the previous item's skip + ntraj), as the reference
// draws ring after ring from one stream (ImpactParameter_Class.F90:202-221).
__host__ __device__ inline bool continues_stream(const cair_work_item* items, int it) {
  if (it == 0 || items[it].skip == 0) return false;
  const cair_work_item& P = items[it - 1];
  return P.seed == items[it].seed && P.skip + P.ntraj == items[it].skip;
}

// One stream, drawn in the reference's order into draws[kDraws * g]: the item `head` and the items
// that continue its stream, each trajectory with its own item's levels and impact-parameter rule.
// A head with skip > 0 (its earlier rings are not among the items) first draws and drops skip
// trajectories under its own rule.  nmol = 1: diatom + atom (SetInitialState_DiatomAtom draws the
// level pick even when state-specific); nmol = 2: diatom + diatom (SetInitialState_DiatomDiatom,
// state-specific: no level draw).  Host and device: the library runs it on the GPU (k_ic_draws).
__host__ __device__ inline void stream_draws(const cair_work_item* items, int nitems, int head, int nmol,
                                             const cair_level* levels, double* draws, int32_t* item_of) {
  Stream st;
  st.seed(items[head].seed);
  auto one = [&](const cair_work_item& W, double* d) {
    if (nmol == 1) st.draw();  // level pick (state-specific: the draw is made and the item's level used)
    for (int mol = 0; mol < nmol; ++mol) {
      const cair_level L = levels[mol == 0 ? W.ilevel : W.ilevel2];
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
      for (int j = 0; j < 4; ++j) d[4 * mol + j] = st.draw();
    }
    d[4 * nmol] = st.draw();
    // a fixed impact parameter (bmax < 0) draws no random number (Collision_Class.F90:1280-1281)
    d[4 * nmol + 1] = W.bmax > 0.0 ? st.draw() : 0.0;
  };
  double skipped[kDraws];
  for (int64_t k = 0; k < items[head].skip; ++k) one(items[head], skipped);
  for (int it = head; it < nitems && (it == head || continues_stream(items, it)); ++it) {
    const cair_work_item& W = items[it];
    for (int64_t k = 0; k < W.ntraj; ++k) {
      const int64_t g = W.first + k;
      one(W, draws + kDraws * g);
      item_of[g] = it;
    }
  }
}

#ifndef CAIR_MODEL_TU  // model-independent: built once, in the API translation unit
// One thread per stream: the thread of an item that continues the previous item's stream has nothing
// to do (the stream's head draws it).
__global__ void k_ic_draws(int nitems, int nmol, const cair_work_item* __restrict__ items,
                           const cair_level* __restrict__ levels, double* __restrict__ draws,
                           int32_t* __restrict__ item_of) {
  int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nitems || continues_stream(items, it)) return;
  stream_draws(items, nitems, it, nmol, levels, draws, item_of);
}
#endif

// The impact parameter of one trajectory (Collision_Class.F90:1276-1296): the ring's input b is
// -bmax; a negative one is sampled by the strata type, a positive one is used as it is.
__host__ __device__ __forceinline__ double impact_parameter(const cair_work_item& W, double u) {
  const double bring = -W.bmax, bmin = -W.bmin;
  if (bring >= 0.0) return bring;
  if (W.b_mode == 1) return sqrt(bmin * bmin + u * (bring * bring - bmin * bmin));
  if (W.b_mode == 2) return bmin + u * (-bring - bmin);
  return -sqrt(u) * bring;
}

// BondLength (StateInitDiatomAtom_Module.F90:543-730): FuncRHS of the radial motion
struct RadialRhs {
  const DevSys& S;
  double xmui, vc_r2;
  __device__ RadialRhs(const DevSys& s, double xm, double vc) : S(s), xmui(xm), vc_r2(vc) {}
  __device__ __forceinline__ void operator()(const double (&y)[2], double (&d)[2]) const {
    double v, dv;
    diat_any<true>(S, y[0], v, dv);
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

// One diatom of masses ma, mb in level L from its four draws (vibphase, rA, rB, rC): BondLength from
// the outer turning point with zero radial velocity and Compute_Coordinates_Velocities
// (StateInitDiatomAtom_Module.F90:543-833); q, qd [dir][atom] relative to the diatom's centre.
__device__ __forceinline__ void diatom_ic(const DevSys& S, const cair_level& L, double ma, double mb,
                                          const double* dr, double (&q)[3][2], double (&qd)[3][2]) {
  const double redmass_d = ma * mb / (ma + mb);
  const double xmui = 1.0 / redmass_d, xmui2 = 0.5 * xmui;
  const double jh = (double)L.jqn + 0.5;
  const double vc_r2 = xmui2 * (jh * jh);
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
  q[0][0] = fa * r * u1; q[1][0] = fa * r * u2; q[2][0] = fa * r * sb * ca;
  q[0][1] = fb * r * u1; q[1][1] = fb * r * u2; q[2][1] = fb * r * sb * ca;
  qd[0][0] = fa * (rdot * u1 + ro_ * w1); qd[1][0] = fa * (rdot * uu1 + ro_ * w2);
  qd[2][0] = fa * (rdot * (sb * ca) + ro_ * sb * sa);
  qd[0][1] = fb * (rdot * u1 + ro_ * w1); qd[1][1] = fb * (rdot * uu1 + ro_ * w2);
  qd[2][1] = fb * (rdot * (sb * ca) + ro_ * sb * sa);
}

// SetPaQ (Collision_Class.F90:1766-1849): p = Tqp^T qdot over the free atoms, q = coordinates; then
// Hamiltonian_0d, SetErrorFactor (both halves from the momenta) and SetInitialPaQ.
template <int MODEL>
__device__ __forceinline__ void finish_ic(const DevSys& S, const cair_work_item& W, const double* qfree,
                                          const double* dqfree, int64_t g, double* __restrict__ paq,
                                          double* __restrict__ paq0, double* __restrict__ erra,
                                          double* __restrict__ H0) {
  using T = Traits<MODEL>;
  double y[T::NE];
  for (int i = 0; i < T::NV; ++i) { y[T::NV + i] = qfree[i]; y[i] = 0.0; }
  for (int ip = 0; ip < T::NV; ++ip)
    for (int i = 0; i < T::NV; ++i) y[i] = y[i] + S.Tqp[ip + 9 * i] * dqfree[ip];
  double rpi[T::NP];
  const double h0 = hamiltonian<MODEL>(S, S.pes[W.ipes], y, rpi);
  double ep = 0.0, eq = 0.0;
  for (int i = 0; i < T::NV; ++i) { ep = ep + y[i] * y[i]; eq = eq + y[i] * y[i]; }
  ep = S.eps * sqrt(ep / T::NV);
  eq = S.eps * sqrt(eq / T::NV);
  for (int i = 0; i < T::NE; ++i) {
    paq[T::NE * g + i] = y[i];
    erra[T::NE * g + i] = i < T::NV ? ep : eq;
    paq0[T::NE * g + i] = i < T::NV ? dqfree[i] : y[i];
  }
  H0[g] = h0;
}

// Diatom (atoms 1, 2) + atom (3): SetIniCondForward (Collision_Class.F90:1065-1211)
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
    const double* dr = draws + kDraws * g;
    const double* m = S.mass;
    double q[3][2], qd[3][2];
    diatom_ic(S, levels[W.ilevel], m[0], m[1], dr, q, qd);
    // CoordVeloc_FreeTotAngMom: Boltzmann energy and the impact parameter
    const double er = boltzmann_er(W.ttra, dr[4]);
    const double b = impact_parameter(W, dr[5]);
    // ComputeCoordinatesVelocities + ShiftCoordinates (the atom sits at the origin of its frame)
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
    double qf[6], dq[6];
    for (int a = 0; a < 2; ++a)
      for (int d = 0; d < 3; ++d) { qf[3 * a + d] = q[d][a]; dq[3 * a + d] = qd[d][a]; }
    finish_ic<MODEL>(S, W, qf, dq, g, paq, paq0, erra, H0);
    bout[g] = b;
    if (key) key[g] = ver;  // initial relative speed: slow collisions run longest
    ipes_out[g] = W.ipes;
  }
}

// Diatom (atoms 1, 2; level ilevel) + diatom (atoms 3, 4; level ilevel2), state-specific:
// SetInitialState_DiatomDiatom (StateInitDiatomDiatom_Module.F90:86-219), then the same relative
// placement, with the projectile's first atom the last free one (SetPaQ, icoord = 0).
template <int MODEL>
__global__ void __launch_bounds__(128) k_sample_ic4(DevSys S, int64_t ntot, const cair_work_item* __restrict__ items,
                                                    const cair_level* __restrict__ levels,
                                                    const double* __restrict__ draws,
                                                    const int32_t* __restrict__ item_of, double* __restrict__ paq,
                                                    double* __restrict__ paq0, double* __restrict__ erra,
                                                    double* __restrict__ H0, double* __restrict__ bout,
                                                    int32_t* __restrict__ ipes_out, double* __restrict__ key) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ntot; g += (int64_t)gridDim.x * blockDim.x) {
    const cair_work_item W = items[item_of[g]];
    const double* dr = draws + kDraws * g;
    const double* m = S.mass;
    double q1[3][2], qd1[3][2], q2[3][2], qd2[3][2];
    diatom_ic(S, levels[W.ilevel], m[0], m[1], dr, q1, qd1);
    diatom_ic(S, levels[W.ilevel2], m[2], m[3], dr + 4, q2, qd2);
    const double er = boltzmann_er(W.ttra, dr[8]);
    const double b = impact_parameter(W, dr[9]);
    const double mt = m[0] + m[1], mp = m[2] + m[3];
    const double redmass = mt * mp / (mt + mp);
    const double fA = -mp / (mt + mp), fB = mt / (mt + mp);
    const double qx1 = fA * W.dinit, qx2 = fB * W.dinit;
    const double ver = sqrt(2.0 * er / redmass);
    const double ratio = b / W.dinit;
    const double verx = -ver * sqrt(1.0 - ratio * ratio), verz = -ver * ratio;
    for (int a = 0; a < 2; ++a) {
      q1[0][a] = q1[0][a] + qx1;
      qd1[0][a] = qd1[0][a] + fA * verx;
      qd1[2][a] = qd1[2][a] + fA * verz;
      q2[0][a] = q2[0][a] + qx2;
      qd2[0][a] = qd2[0][a] + fB * verx;
      qd2[2][a] = qd2[2][a] + fB * verz;
    }
    double qf[9], dq[9];
    for (int d = 0; d < 3; ++d) {
      qf[d] = q1[d][0]; dq[d] = qd1[d][0];
      qf[3 + d] = q1[d][1]; dq[3 + d] = qd1[d][1];
      qf[6 + d] = q2[d][0]; dq[6 + d] = qd2[d][0];
    }
    finish_ic<MODEL>(S, W, qf, dq, g, paq, paq0, erra, H0);
    bout[g] = b;
    if (key) key[g] = ver;
    ipes_out[g] = W.ipes;
  }
}

// Analyse the initial and final points of each trajectory and assemble its output row
// (Integrator_Class.F90:884-933).
#ifndef CAIR_MODEL_TU  // model-independent: built once, in the API translation unit
template <int NA>
__global__ void __launch_bounds__(128) k_results(DevSys S, FsArgs F, int64_t n, const double* __restrict__ paq0,
                                                 const double* __restrict__ paq, const double* __restrict__ H0,
                                                 const double* __restrict__ H, const double* __restrict__ t,
                                                 const int32_t* __restrict__ status,
                                                 const int32_t* __restrict__ iste,
                                                 const int32_t* __restrict__ irej,
                                                 const int32_t* __restrict__ item_of,
                                                 const cair_work_item* __restrict__ items,
                                                 cair_traj_result* __restrict__ out) {
  constexpr int NV = 3 * (NA - 1), NE = 2 * NV;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    double v[NE];
    // ApplyTransformation: momenta -> velocities
    for (int i = 0; i < NV; ++i) {
      double a = 0.0;
      for (int j = 0; j < NV; ++j) a = a + S.Tpq[i + 9 * j] * paq[NE * k + j];
      v[i] = a;
    }
    for (int i = NV; i < NE; ++i) v[i] = paq[NE * k + i];
    cair_traj_point pi, pf;
    analyze<NA>(S, F, paq0 + NE * k, pi);
    analyze<NA>(S, F, v, pf);
    cair_traj_result r;
    const int it = item_of ? item_of[k] : 0;
    r.item = it;
    r.idx = item_of ? (items[it].skip + k - items[it].first + 1) : (k + 1);
    r.ipes = item_of ? items[it].ipes : 0;
    r.status = status[k];
    r.iste = iste[k];
    r.irej = irej[k];
    r.pad = 0;
    r.bmax = item_of ? fabs(items[it].bmax) : 0.0;
    r.b = pi.b;
    r.j_i = pi.mol[0].angmom;
    r.v_i = pi.mol[0].viba;
    r.j_f = pf.mol[0].angmom;
    r.v_f = pf.mol[0].viba;
    if (NA == 3) {
      r.arr_i = pi.mol[0].ipair * 16.0 + (double)pi.mol[0].itype + 0.5;
      r.arr_f = pf.mol[0].ipair * 16.0 + (double)pf.mol[0].itype + 0.5;
      r.j2_i = r.v2_i = r.j2_f = r.v2_f = 0.0;
    } else {
      r.arr_i = pi.mol[0].ipair * 16.0 + (double)pi.mol[0].itype + 4.0 * pi.mol[1].itype + 0.5;
      r.arr_f = pf.mol[0].ipair * 16.0 + (double)pf.mol[0].itype + 4.0 * pf.mol[1].itype + 0.5;
      r.j2_i = pi.mol[1].angmom;
      r.v2_i = pi.mol[1].viba;
      r.j2_f = pf.mol[1].angmom;
      r.v2_f = pf.mol[1].viba;
    }
    r.t = t[k];
    r.dH = H[k] - H0[k];
    out[k] = r;
  }
}
#endif

}  // namespace cair
