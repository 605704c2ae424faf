"""CPU tests of the oracle (the CPU restatement of the reference path) -- its pins.

The reference ships no golden values for these surfaces or the integrator, so the oracle is
pinned by: finite-difference gradients, permutation symmetry and dissociation limits of each
surface; an independent big-integer restatement of the random-number generator; the inverse
of the Boltzmann energy CDF; energy conservation of the integrator; and the shipped level lists
read as known-answer tests of the final-state chain (turning points and action -> v + 1/2).
"""
import numpy as np
import pytest

from coarseair_gb300 import systems


def _cfgs():
    return [systems.o3_config(), systems.n3_config(), systems.o4_config(), systems.n4_config()]


def _random_geometry(rng, natoms, n):
    """Random Cartesian coordinates of the NAtoms-1 free atoms with pair distances 1.6..5 bohr."""
    out = []
    while len(out) < n:
        q = rng.uniform(-2.5, 2.5, size=3 * (natoms - 1))
        out.append(q)
    return np.array(out)


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_surface_gradient_matches_finite_differences(oracle_lib, idx):
    from oracle import Oracle
    cfg = _cfgs()[idx]
    o = Oracle(cfg)
    rng = np.random.default_rng(7 + idx)
    Q = _random_geometry(rng, cfg.natoms, 40)
    R, Qall = o.rp(Q)
    keep = np.all((R > 1.6) & (R < 6.0), axis=1)
    R, Qall = R[keep][:8], Qall[keep][:8]
    assert R.shape[0] >= 4
    V, g, _ = o.compute(R, Qall)
    # the 430-term O4 fit carries ~1e-12 Eh of cancellation noise; h = 2e-3 keeps the
    # fourth-order difference's round-off and truncation both near 1e-9
    h = 2e-3
    for i in range(cfg.npairs):
        def f(dx):
            Rs = R.copy()
            Rs[:, i] += dx
            return o.potential(Rs)
        # fourth-order central difference
        fd = (8 * (f(h) - f(-h)) - (f(2 * h) - f(-2 * h))) / (12 * h)
        scale = np.maximum(np.abs(g).max(axis=1), 1e-3)
        assert np.all(np.abs(fd - g[:, i]) / scale < 1e-8), (i, fd, g[:, i])


@pytest.mark.parametrize("idx", [0, 1])
def test_cartesian_forces_match_finite_differences(oracle_lib, idx):
    from oracle import Oracle
    cfg = _cfgs()[idx]
    o = Oracle(cfg)
    Q = np.array([[0.3, 0.2, -0.1, 2.5, 0.1, 0.05], [-1.0, 0.4, 0.3, 1.2, -0.2, 0.7]])
    R, Qall = o.rp(Q)
    _, _, m = o.compute(R, Qall)
    h = 1e-4
    for i in range(6):
        def f(dx):
            Qs = Q.copy()
            Qs[:, i] += dx
            return o.potential(o.rp(Qs)[0])
        fd = (8 * (f(h) - f(-h)) - (f(2 * h) - f(-2 * h))) / (12 * h)
        assert np.all(np.abs(fd - m[:, i]) < 1e-8 * np.abs(m).max(axis=1) + 1e-11), (i, fd, m[:, i])


@pytest.mark.parametrize("idx", [0, 1])
def test_three_atom_surfaces_are_permutation_invariant(oracle_lib, idx):
    """Identical atoms: swapping atoms 1 and 2 maps the pairs (12, 13, 23) to (12, 23, 13)."""
    from oracle import Oracle
    o = Oracle(_cfgs()[idx])
    R = np.array([[2.1, 2.9, 3.7], [2.3, 2.4, 4.0], [3.0, 3.1, 3.2]])
    v = o.potential(R)
    for perm in ([0, 2, 1], [2, 1, 0], [1, 0, 2], [1, 2, 0], [2, 0, 1]):
        assert np.allclose(o.potential(R[:, perm]), v, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("idx", [2, 3])
def test_four_atom_surface_is_permutation_invariant(oracle_lib, idx):
    """O4, N4: swapping atoms 1 <-> 2 maps pairs (12,13,14,23,24,34) -> (12,23,24,13,14,34)."""
    from oracle import Oracle
    o = Oracle(_cfgs()[idx])
    R = np.array([[2.3, 3.1, 4.2, 3.6, 3.9, 2.4], [2.2, 5.0, 5.5, 4.7, 5.2, 2.3]])
    v = o.potential(R)
    assert np.allclose(o.potential(R[:, [0, 3, 4, 1, 2, 5]]), v, rtol=1e-11, atol=1e-12)
    # atoms 3 <-> 4: (12,13,14,23,24,34) -> (12,14,13,24,23,34)
    assert np.allclose(o.potential(R[:, [0, 2, 1, 4, 3, 5]]), v, rtol=1e-11, atol=1e-12)
    # molecules swapped (1,2) <-> (3,4): (12,13,14,23,24,34) -> (34,13,23,14,24,12)
    assert np.allclose(o.potential(R[:, [5, 1, 3, 2, 4, 0]]), v, rtol=1e-11, atol=1e-12)


def test_n4_reduces_to_n3_with_a_distant_atom(oracle_lib):
    """N4 UMN with atom 4 at 10^3 bohr from the others is the N3 UMN fit (the N3 surface is the N4
    PIP with those pairs pinned at 10^3 bohr) plus the three far N2 diatomic terms."""
    from oracle import Oracle
    L = oracle_lib.lib()
    o4, o3 = Oracle(systems.n4_config()), Oracle(systems.n3_config())
    for r in ([2.1, 2.9, 3.7], [2.07, 4.0, 5.5]):
        v3 = o3.potential(np.array([r]))[0]
        v4 = o4.potential(np.array([[r[0], r[1], 1.0e3, r[2], 1.0e3, 1.0e3]]))[0]
        assert abs(v4 - (v3 + 3 * L.orc_diat_V(2, 1.0e3))) < 1e-12


def test_n3_dissociation_limit(oracle_lib):
    """With atom 3 far away the N3 surface is the N2 diatomic plus the constant totdiss term."""
    from oracle import Oracle
    L = oracle_lib.lib()
    o = Oracle(systems.n3_config())
    for r in (1.8, 2.07, 2.6):
        v = o.potential(np.array([[r, 60.0, 60.0 + r]]))[0]
        vd = L.orc_diat_V(2, r) + 2 * L.orc_diat_V(2, 60.0)
        assert abs(v - (vd + 457.4 * 0.159360144e-2)) < 1e-10


def test_o3_dissociation_limit(oracle_lib):
    from oracle import Oracle
    L = oracle_lib.lib()
    o = Oracle(systems.o3_config())
    for r in (2.0, 2.28, 3.0):
        v = o.potential(np.array([[r, 60.0, 60.0 + r]]))[0]
        vd = L.orc_diat_V(1, r) + L.orc_diat_V(1, 60.0) + L.orc_diat_V(1, 60.0 + r)
        assert abs(v - vd) < 1e-10


def _o3nn_numpy(coef, R):
    """Independent numpy restatement of the O3 NN network part (O3_NN_PES_Class.F90): the Compute
    features and network with its gradient by the chain rule, and the Potential variant (three
    scaled features, W1's storage read as a 3 x NHL1 matrix by dgemm with leading dimension 3)."""
    h1, h2 = int(coef[0]), int(coef[1])
    lam, re_ = coef[2], coef[3]
    mean, sd, ysc = coef[4:7], coef[7:10], coef[10]
    q = 11
    W1f = coef[q:q + 6 * h1]; q += 6 * h1
    b1 = coef[q:q + h1]; q += h1
    W2 = coef[q:q + h1 * h2].reshape(h2, h1).T; q += h1 * h2
    b2 = coef[q:q + h2]; q += h2
    W3 = coef[q:q + h2]; q += h2
    b3 = coef[q]
    W1 = W1f.reshape(h1, 6).T
    p = np.exp(-lam * (R - re_))
    p1, p2, p3 = p.T
    G = np.stack([p1 * p2 + p2 * p3 + p3 * p1, p1 * p2 * p3,
                  p1 * p1 * p2 + p1 * p2 * p2 + p2 * p2 * p3 + p2 * p3 * p3 + p1 * p1 * p3 + p1 * p3 * p3,
                  p1 ** 3 * p2 + p1 * p2 ** 3 + p2 ** 3 * p3 + p2 * p3 ** 3 + p1 ** 3 * p3 + p1 * p3 ** 3,
                  p1 * p2 * p3 * (p1 + p2 + p3),
                  p1 * p1 * p2 * p2 + p2 * p2 * p3 * p3 + p1 * p1 * p3 * p3], axis=1)
    y1 = np.tanh(G @ W1 + b1)
    y2 = np.tanh(y1 @ W2 + b2)
    V = (y2 @ W3 + b3 - ysc) / 27.2113839712790
    # chain rule: dV/dG then dG/dp by symbolic partials, dp/dR = -lam p
    d2 = W3 * (1 - y2 ** 2)
    d1 = (d2 @ W2.T) * (1 - y1 ** 2)
    dVdG = d1 @ W1.T
    dGdp = np.zeros((len(R), 6, 3))
    P = [p1, p2, p3]
    for a in range(3):
        b, c = [x for x in range(3) if x != a]
        pa, pb, pc = P[a], P[b], P[c]
        dGdp[:, 0, a] = pb + pc
        dGdp[:, 1, a] = pb * pc
        dGdp[:, 2, a] = 2 * pa * (pb + pc) + pb * pb + pc * pc
        dGdp[:, 3, a] = 3 * pa * pa * (pb + pc) + pb ** 3 + pc ** 3
        dGdp[:, 4, a] = pb * pc * (2 * pa + pb + pc)
        dGdp[:, 5, a] = 2 * pa * (pb * pb + pc * pc)
    dV = np.einsum("ni,nia->na", dVdG, dGdp) * (-lam * p) / 27.2113839712790
    Gp = np.stack([p1 * p2 + p2 * p3 + p3 * p1, p1 * p2 * p3,
                   p1 * p2 * (p1 + p2) + p2 * p3 * (p2 + p3) + p3 * p1 * (p3 + p1)], axis=1)
    Gp = (Gp - mean) / sd
    W1p = W1f[:3 * h1].reshape(h1, 3).T
    Vp = (np.tanh(np.tanh(Gp @ W1p + b1) @ W2 + b2) @ W3 + b3 - ysc) / 27.2113839712790
    return V, dV, Vp


def test_o3nn_surface_pins(oracle_lib):
    """O3 NN: Compute and Potential against an independent numpy restatement, the analytic
    gradient against finite differences of Compute's energy, permutation invariance."""
    from oracle import Oracle
    L = oracle_lib.lib()
    cfg = systems.o3nn_config()
    o = Oracle(cfg)
    rng = np.random.default_rng(11)
    Q = _random_geometry(rng, 3, 200)
    R, Qall = o.rp(Q)
    keep = np.all((R > 1.6) & (R < 8.0), axis=1)
    R, Qall = R[keep][:40], Qall[keep][:40]
    V, g, _ = o.compute(R, Qall)
    Vd = np.array([[L.orc_diat_V(1, r) for r in row] for row in R]).sum(axis=1)
    dVd = np.zeros_like(R)
    import ctypes
    for n, row in enumerate(R):
        for i, r in enumerate(row):
            v, dv = ctypes.c_double(), ctypes.c_double()
            L.orc_diat_VdV(1, r, ctypes.byref(v), ctypes.byref(dv))
            dVd[n, i] = dv.value
    Vn, dVn, Vpn = _o3nn_numpy(cfg.surfaces[0].coef, R)
    assert np.allclose(V, Vn + Vd, rtol=1e-12, atol=1e-13)
    assert np.allclose(g, dVn + dVd, rtol=1e-10, atol=1e-12)
    assert np.allclose(o.potential(R), Vpn + Vd, rtol=1e-12, atol=1e-13)
    # the two energy routines of the reference differ (Potential is not Compute's energy)
    assert np.max(np.abs(o.potential(R) - V)) > 1e-3
    h = 1e-4
    for i in range(3):
        def f(dx):
            Rs = R.copy()
            Rs[:, i] += dx
            return o.compute(Rs, Qall)[0]
        fd = (8 * (f(h) - f(-h)) - (f(2 * h) - f(-2 * h))) / (12 * h)
        assert np.all(np.abs(fd - g[:, i]) < 1e-8 * np.maximum(np.abs(g).max(axis=1), 1e-3))
    for perm in ([0, 2, 1], [2, 1, 0], [1, 0, 2]):
        Vp, _, _ = o.compute(R[:, perm], Qall)
        assert np.allclose(Vp, V, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("sample", [1, 17, 50])
def test_o3bnn_surface_pins(oracle_lib, sample):
    """O3 BNN posterior samples (BNN_PES_Class.F90): Compute and Potential against the numpy
    restatement of the NN networks taken through VExp = exp(v + Noise) (the gradient gains the factor
    VExp), the gradient against finite differences of Compute's energy, permutation invariance."""
    import ctypes
    from oracle import Oracle
    L = oracle_lib.lib()
    cfg = systems.o3bnn_config(samples=[sample])
    coef = cfg.surfaces[0].coef
    h1, h2 = int(coef[0]), int(coef[1])
    assert coef.size == 13 + 7 * h1 + h1 * h2 + 2 * h2
    noise, ysc = coef[-1], coef[10]
    o = Oracle(cfg)
    rng = np.random.default_rng(13 + sample)
    Q = _random_geometry(rng, 3, 200)
    R, Qall = o.rp(Q)
    keep = np.all((R > 1.6) & (R < 8.0), axis=1)
    R, Qall = R[keep][:40], Qall[keep][:40]
    V, g, _ = o.compute(R, Qall)
    Vd, dVd = np.zeros(len(R)), np.zeros_like(R)
    for n, row in enumerate(R):
        for i, r in enumerate(row):
            v, dv = ctypes.c_double(), ctypes.c_double()
            L.orc_diat_VdV(1, r, ctypes.byref(v), ctypes.byref(dv))
            Vd[n] += v.value
            dVd[n, i] = dv.value
    Vn, dVn, Vpn = _o3nn_numpy(coef[:-1], R)
    ev = 27.2113839712790
    vexp = np.exp(Vn * ev + ysc + noise)
    assert np.allclose(V, (vexp - ysc) / ev + Vd, rtol=1e-12, atol=1e-13)
    assert np.allclose(g, vexp[:, None] * dVn + dVd, rtol=1e-10, atol=1e-12)
    assert np.allclose(o.potential(R), (np.exp(Vpn * ev + ysc + noise) - ysc) / ev + Vd, rtol=1e-12, atol=1e-13)
    assert np.max(np.abs(o.potential(R) - V)) > 1e-4
    h = 1e-4
    for i in range(3):
        def f(dx):
            Rs = R.copy()
            Rs[:, i] += dx
            return o.compute(Rs, Qall)[0]
        fd = (8 * (f(h) - f(-h)) - (f(2 * h) - f(-2 * h))) / (12 * h)
        assert np.all(np.abs(fd - g[:, i]) < 1e-8 * np.maximum(np.abs(g).max(axis=1), 1e-3))
    for perm in ([0, 2, 1], [2, 1, 0], [1, 0, 2]):
        Vp, _, _ = o.compute(R[:, perm], Qall)
        assert np.allclose(Vp, V, rtol=1e-12, atol=1e-13)


def _rand12_bigint(digits):
    """Independent restatement of rand12 (RandomVector_Module.F90:166-229) on base-256 digits."""
    ia = [45, 127, 149, 76, 45, 244, 81, 88]
    idd = [0] * 16
    for j in range(8):
        for i in range(8 - j):
            k = j + i
            ip = ia[j] * digits[i]
            while True:
                ip = ip + idd[k]
                idd[k] = ip % 256
                ip = ip // 256
                if ip == 0 or k == 7:
                    break
                k += 1
    digits[:] = idd[:8]
    r = float(digits[0])
    for i in range(1, 8):
        r = float(digits[i]) + r * 3.90625e-3
    return r * 3.90625e-3


@pytest.mark.parametrize("seed", [1, 2, 3, 12345])
def test_rng_matches_independent_base256_restatement(oracle_lib, seed):
    import ctypes
    L = oracle_lib.lib()
    st = oracle_lib.OrcRng()
    L.orc_rng_seed(ctypes.byref(st), seed)
    s = seed - 1 if seed % 2 == 0 else seed
    digits = [(s >> (8 * i)) & 0xFF for i in range(8)]
    table = [_rand12_bigint(digits) for _ in range(100)]
    for _ in range(300):
        i = int(99.0 * table[99]) + 1
        expect = table[99]
        table[99] = table[i - 1]
        table[i - 1] = _rand12_bigint(digits)
        assert L.orc_rng_draw(ctypes.byref(st)) == expect


def test_boltzmann_energy_inverts_flux_weighted_cdf(oracle_lib):
    L = oracle_lib.lib()
    kelvin_to_hartree = 1.0 / 3.1577513e5
    for u in (0.05, 0.3, 0.5, 0.77, 0.95):
        er = L.orc_boltzmann_er(10000.0, u)
        x = er / (10000.0 * kelvin_to_hartree)
        assert abs((1 - (1 + x) * np.exp(-x)) - u) < 1e-4


# reference masses of the shipped level lists (input/O3/UMN/input/CoarseAIR.inp, input/N3/...)
REF_MASS = {"O2": 29148.94559, "N2": 25526.04298}
DIAT = {"O2": 1, "N2": 2}


# (max |V_eff(ri) - V_eff(ro)|, max |v + 1/2 - action/2pi|, median of the latter, offset spread)
KAT_TOL = {"O2": (2e-4, 0.05, 0.005, 3e-4), "N2": (1e-3, 0.25, 0.01, 6e-4)}


@pytest.mark.parametrize("mol", ["N2", "O2"])
def test_level_list_known_answers(oracle_lib, mol):
    """Shipped level lists as known answers for the final-state chain.

    The lists give (v, J) with turning points ri, ro.  On the surface's diatomic potential the
    effective potential must agree at ri and ro, each list's energy zero differs from the
    potential's by one constant, and the semiclassical action over [ri, ro] divided by 2 pi is
    v + 1/2 (MolecularState_Class.F90:297).  The lists were generated with earlier versions of
    the diatomic potentials (the O2 list puts the zero at the well bottom, the N2 list comes
    from another fit), so these hold to the tolerances of KAT_TOL, not to rounding.
    """
    L = oracle_lib.lib()
    lv = systems.load_levels(mol)
    mu = REF_MASS[mol] / 2.0
    rows = lv[np.random.default_rng(11).choice(len(lv), 300, replace=False)]
    rows = rows[rows["egam"] == 0.0]
    dv, off, dvib = [], [], []
    for r in rows:
        vc_r2 = 0.5 / mu * (r["jqn"] + 0.5) ** 2
        vri = L.orc_diat_V(DIAT[mol], r["ri"]) + vc_r2 / r["ri"] ** 2
        vro = L.orc_diat_V(DIAT[mol], r["ro"]) + vc_r2 / r["ro"] ** 2
        e = 0.5 * (vri + vro)
        dv.append(abs(vri - vro))
        off.append(r["eint"] - e)
        act = L.orc_action_integral(DIAT[mol], r["ri"], r["ro"], vc_r2, e, 50, 2 * mu)
        dvib.append(abs(act * 0.5 / np.pi - (r["vqn"] + 0.5)))
    tol = KAT_TOL[mol]
    assert max(dv) < tol[0]
    assert max(dvib) < tol[1] and np.median(dvib) < tol[2]
    assert max(off) - min(off) < tol[3]


def test_initial_conditions_recover_sampled_level(oracle_lib):
    """IC sampler (BondLength, orientation) + FindState on PaQ0 returns the sampled (v, J)."""
    from oracle import Oracle
    cfg = systems.n3_config(mass_amu=REF_MASS["N2"] / systems.AMU_TO_AU)
    o = Oracle(cfg)
    lv = systems.load_levels("N2")
    for v, j in ((0, 0), (3, 20), (10, 45)):
        sel = lv[(lv["vqn"] == v) & (lv["jqn"] == j)]
        ic = o.sample_ics(6, sel)
        fs = o.analyze(ic["paq0"])
        for f in fs:
            assert f["ipair"] == 1
            assert abs(f["viba"] - (v + 0.5)) < 2e-2  # list ro vs this potential (see KAT_TOL)
            assert abs(f["angmom"] - (j + 0.5)) < 1e-6


def test_diatom_diatom_initial_conditions_recover_both_levels(oracle_lib):
    """Diatom + diatom sampler (SetInitialState_DiatomDiatom for each molecule, relative placement
    with atom 4 eliminated) + the four-atom analysis on PaQ0: molecule 1 is pair 1-2 in the target's
    level, molecule 2 the opposite pair 3-4 in the projectile's, and the impact parameter and
    relative kinetic energy are the sampled ones."""
    from oracle import Oracle
    cfg = systems.o4_config(mass_amu=REF_MASS["O2"] / systems.AMU_TO_AU)
    o = Oracle(cfg)
    lv = systems.load_levels("O2")
    for (v1, j1), (v2, j2) in (((0, 1), (0, 1)), ((2, 15), (5, 33))):
        a = lv[(lv["vqn"] == v1) & (lv["jqn"] == j1)][0]
        b = lv[(lv["vqn"] == v2) & (lv["jqn"] == j2)][0]
        ic = o.sample_ics4(5, a, b, ttra=10000.0, bmax=8.0, dinit=18.0, seed=7)
        for k, f in enumerate(o.analyze(ic["paq0"])):
            assert (f["ipair"], f["ipair1"]) == (1, 6)
            assert abs(f["angmom"] - (j1 + 0.5)) < 1e-6 and abs(f["angmom1"] - (j2 + 0.5)) < 1e-6
            assert abs(f["viba"] - (v1 + 0.5)) < 2e-2 and abs(f["viba1"] - (v2 + 0.5)) < 2e-2
            assert abs(f["b"] - ic["b"][k]) < 1e-9
            # kinetic energy of the two centres of mass = the sampled relative translational energy
            assert abs(f["xkin"] - ic["er"][k]) < 1e-10 * ic["er"][k]


def test_integration_conserves_energy(oracle_lib):
    from oracle import Oracle
    cfg = systems.o3_config()
    o = Oracle(cfg)
    lv = systems.load_levels("O2")
    sel = lv[(lv["vqn"] == 0) & (lv["jqn"] == 1)]
    ic = o.sample_ics(6, sel)
    res = o.integrate(ic["paq"], ic["erra"])
    assert np.all(res["status"] == 0)
    assert np.max(np.abs(res["H"] - ic["H0"])) < cfg.ham_abs_tol


def test_statistics_known_answers(oracle_lib):
    """Histogram statistics of six hand-made rows (Statistics_Class.F90): J folded by even/oddness
    within the initial arrangement, arrangement change, dissociated v < 0; Cross = pi bmax^2 n/N,
    CrossSD = sqrt(w (1 - w) A^2 / N); Boltzmann mean velocity in cm^3/s per bohr^2."""
    import oracle
    qini = np.array([[10.5, 0.5, 16.5]] * 6)
    qfin = np.array([[10.5, 0.5, 16.5], [12.4, 0.6, 16.5], [11.6, 1.2, 16.5], [8.5, 0.5, 32.5],
                     [20.0, -1.0, 18.5], [10.5, 0.5, 16.5]])
    res, ini = oracle.statistics(np.full(6, 7.0), np.linspace(1, 6, 6), qini, qfin, pres=(1, 0, 0))
    assert ini == (10, 0, 16)
    got = {r[0]: r[1:] for r in res}
    assert set(got) == {(10, 0, 16), (12, 0, 16), (12, 1, 16), (8, 0, 32), (20, -2, 18)}
    area = np.pi * 49.0
    for fs, (n, cross, sd) in got.items():
        w = n / 6.0
        assert n == (2 if fs == (10, 0, 16) else 1)
        assert cross == pytest.approx(area * w, rel=1e-15)
        assert sd == pytest.approx(np.sqrt(w * (1 - w) * area * area / 6.0), rel=1e-15)
    xmu = 1822.888486209 * 14.0067 * 2 / 3
    vp = np.sqrt(2 * 10000.0 / 3.1577513e5 / xmu)
    assert oracle.mean_velocity(10000.0, xmu) == pytest.approx(2 / np.sqrt(np.pi) * vp * 4.134137e16 * 0.5291771e-8 ** 3,
                                                               rel=1e-14)


SCATTERING_RINGS = ([-0.25, -0.5, -1.0, -2.5, -4.0, -7.55], [1, 1, 1, 1, 1, 1])  # CoarseAIR_Scattering.inp:166-178
RINGS_EXAMPLE = ([-6.0, -14.0], [1, 99])                                          # CoarseAIR_Scattering.inp:181-186


def test_impact_parameter_rings_split_like_the_reference(oracle_lib):
    """InitializeImpactParameter on the reference's own stratified inputs: equal weights give
    int(N/6) per ring with the remainder in the first; api.ring_entries (the product's helper) and
    the oracle's restatement agree on counts, stream offsets and (bmin, b) for every weight set."""
    import oracle
    from coarseair_gb300 import api
    assert [e[2] for e in api.ring_entries(0, 0, 100, 1, 1e4, 15.0, *SCATTERING_RINGS)] == [20, 16, 16, 16, 16, 16]
    assert [e[2] for e in api.ring_entries(0, 0, 100, 1, 1e4, 15.0, *RINGS_EXAMPLE, strata="Rings")] == [1, 99]
    rng = np.random.default_rng(3)
    for _ in range(50):
        nr = int(rng.integers(1, 7))
        bring = list(-rng.uniform(0.5, 9.0, nr))
        ntring = [int(x) for x in rng.integers(1, 40, nr)]
        n = int(rng.integers(nr, 5000))
        ent = api.ring_entries(0, 0, n, 1, 1e4, 15.0, bring, ntring)
        itm = oracle.impact_rings(n, bring, ntring)
        assert [e[10] + e[2] for e in ent] == itm
        for e in ent:
            for idx in (e[10] + 1, e[10] + e[2]):
                if e[2] == 0:
                    continue
                bmin, b = oracle.impact_ring_of(idx, bring, itm)
                assert (-e[5], -e[9]) == (b, bmin)


@pytest.mark.parametrize("mode,rings", [(0, SCATTERING_RINGS), (1, RINGS_EXAMPLE), (2, RINGS_EXAMPLE)])
def test_stratified_impact_parameters_stay_in_their_strata(oracle_lib, mode, rings):
    """Collision_Class.F90:1276-1296 on the oracle's stream: Circles samples each ring's whole disc,
    Rings the annulus between the previous ring and this one, Segments b = bmin + U (|b| - bmin)
    with the previous ring's signed input value."""
    import oracle
    from oracle import Oracle
    from coarseair_gb300 import systems
    o = Oracle(systems.n3_config())
    lv = systems.load_levels("N2")[[5]]
    lvo = np.zeros(1, dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax", "tau",
                                                   "ri", "ro", "rlim")])
    for c in lvo.dtype.names:
        lvo[c] = lv[c] if c in lv.dtype.names else 0.0
    n = 120
    ic = o.sample_ics(n, lvo, seed=7, ttra=1e4, dinit=15.0, rings=(rings[0], rings[1], mode))
    itm = oracle.impact_rings(n, *rings)
    for k in range(n):
        bmin, b = oracle.impact_ring_of(k + 1, rings[0], itm)
        lo, hi = {0: (0.0, -b), 1: (-bmin, -b), 2: (bmin, -b)}[mode]
        assert lo - 1e-12 <= ic["b"][k] <= hi + 1e-12


def _umn_originals():
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "umn_originals.json")) as f:
        return json.load(f)


# golden key -> (system config with that one surface, the surface, totdiss the oracle adds, diatomic id)
def _umn_case(key):
    if key.startswith("O4_"):
        s = systems.load_o4_umn("UMN_" + key[3:])
        cfg = systems.o4_config()
        cfg.surfaces = [s]
        return cfg, s, 0.0, 1
    if key == "O3_25A1":
        s = systems.load_o3_umn("UMN_25A1")
        cfg = systems.o3_config()
        cfg.surfaces = [s]
        return cfg, s, 0.0, 1
    if key == "N4":
        cfg = systems.n4_config()
        return cfg, cfg.surfaces[0], 457.4, 2
    cfg = systems.n3_config()
    return cfg, cfg.surfaces[0], 457.4, 2


@pytest.mark.parametrize("key", ["O4_Singlet", "O4_Triplet", "O4_Quintet", "N4", "N3", "O3_25A1"])
def test_umn_surfaces_against_the_original_umn_modules(oracle_lib, key):
    """The UMN surfaces against the original UMN Fortran modules the reference ships beside its fits
    (golden values made by tests/golden/make_umn_originals.py): the same coefficients and MEG
    parameters as the fit files the reference reads (the N3 coefficients it keeps inline equal the
    N4 module's), the same polynomial bases, and the oracle's sum C(i) B(i) equal to the module's own
    statements evaluated at the same geometries, to the rounding scale of that sum (N3: the N4
    module at the same three distances with the pairs to the fourth atom at 10^3 bohr)."""
    import ctypes
    from oracle import Oracle
    g = _umn_originals()[key]
    cfg, s, totdiss, diat = _umn_case(key)
    assert np.array_equal(s.coef, np.array(g["C"]))
    if key not in ("N4", "N3"):   # the N3/N4 classes hold a, ab, re inline (1, 1.5, 1.098), as the module does
        assert (s.a, s.ab, s.ra, s.rb) == (g["a"], g["ab"], g["ra"], g["rb"])
    else:
        assert (g["a"], g["ab"], g["ra"], g["rb"], g["totdiss"]) == (1.0, 1.5, 1.098, 1.098, totdiss)
    L = oracle_lib.lib()
    L.orc_const.restype, L.orc_const.argtypes = ctypes.c_double, [ctypes.c_char_p]
    kcm = L.orc_const(b"Kcm_To_Hartree")
    assert kcm == g["Econv"] and L.orc_const(b"B_To_Ang") == g["Cconv"]
    o = Oracle(cfg)
    R = np.array(g["R3_bohr"] if key == "N3" else g["R_bohr"])
    V = o.potential(R)
    vd = np.array([sum(L.orc_diat_V(diat, r) for r in row) for row in R])
    sum_cb = (V - vd) / kcm - totdiss
    ref, scale = np.array(g["sum_cb_kcal"]), np.array(g["abs_sum_cb_kcal"])
    depth = 630 if key.startswith("O4") else 110
    assert np.all(np.abs(sum_cb - ref) <= 2 * depth * 1.1102230246251565e-16 * (scale + totdiss) + 1e-9)


def test_diatomics_against_the_original_umn_modules(oracle_lib):
    """The O2 and N2 UMN diatomics (the oracle's, as the reference's O2_UMN and N2_UMN_ForN4 classes have
    them) against ev2gm2 of the original modules, constants read from the modules.  O2: equal to
    rounding (its Gaussian terms reach ~53 Eh) in the units the reference's class keeps, and within
    1e-6 relative of the module's kcal/mol values, the gap being the module's autoang and autokcal
    against the reference's B_To_Ang and hartree.  N2: the module's kcal/mol values x Econv to 1e-9
    relative (the reference's class writes re^4 as the literal 1.4534810048)."""
    g = _umn_originals()
    L = oracle_lib.lib()
    o2 = g["O2"]
    r = np.array(o2["r_bohr"])
    v = np.array([L.orc_diat_V(1, x) for x in r])
    assert np.all(np.abs(v - np.array(o2["v_hartree_reference_units"])) <= 2e-14)
    vk = np.array(o2["v_kcal"]) * 0.159360144e-2
    assert np.all(np.abs(v - vk) <= 1e-6 * np.maximum(np.abs(vk), 1e-2))
    n2 = g["N2"]
    v = np.array([L.orc_diat_V(2, x) for x in r])
    vk = np.array(n2["v_kcal"]) * 0.159360144e-2
    assert np.all(np.abs(v - vk) <= 1e-9 * np.maximum(np.abs(vk), 1e-2))


def test_ring_entries_edge_cases():
    """One ring, a zero-weight ring (no trajectories, the stream offsets unchanged), a fixed ring, and
    the refusals (negative weights, a weight per ring)."""
    from coarseair_gb300 import api
    one = api.ring_entries(3, 1, 50, 7, 1e4, 15.0, [-6.0], [1])
    assert one == [(3, 1, 50, 7, 1e4, 6.0, 15.0, 0, 0, 0.0, 0)]
    ent = api.ring_entries(0, 0, 10, 7, 1e4, 15.0, [-2.0, -4.0, -6.0], [1, 0, 1])
    assert [e[2] for e in ent] == [5, 0, 5] and [e[10] for e in ent] == [0, 5, 5]
    items = api.work_items(ent)
    assert list(items["first"]) == [0, 5, 5] and list(items["skip"]) == [0, 5, 5]
    fixed = api.ring_entries(0, 0, 4, 7, 1e4, 15.0, [2.5], [1])
    assert fixed[0][5] == -2.5
    with pytest.raises(ValueError):
        api.ring_entries(0, 0, 10, 7, 1e4, 15.0, [-2.0, -4.0], [1, -1])
    with pytest.raises(ValueError):
        api.ring_entries(0, 0, 10, 7, 1e4, 15.0, [-2.0, -4.0], [1])
