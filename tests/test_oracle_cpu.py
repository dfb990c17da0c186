"""CPU checks of the oracle: known answers from the Java SE specification and from physics.

The reference ships no tests or golden vectors; these pin the oracle instead.
"""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi
from starfish_gb300 import workloads as W


def test_java_random_known_values():
    # java.util.Random(0).nextDouble() sequence (Java SE API LCG; widely published values)
    r = O.jrandom_doubles(0, 2)
    assert r[0] == pytest.approx(0.730967787376657, abs=1e-15)
    assert r[1] == pytest.approx(0.24053641567148587, abs=1e-15)
    assert O.jrandom_doubles(42, 1)[0] == pytest.approx(0.7275636800328681, abs=1e-15)


def test_sampler_moments():
    # Utils.SampleMaxw3D: sum of 12 uniforms, scaled by v_th * 1.2 * sqrt(1/2)
    v = O.sample_maxw3d(1, 200000, 1000.0)
    sig = 1000.0 * 1.2 * np.sqrt(0.5)
    assert abs(v.mean()) < 5 * sig / np.sqrt(v.size)
    assert v.std() == pytest.approx(sig, rel=5e-3)
    s = O.sample_maxw_speed(2, 100000, 1000.0)
    # Maxwell speed distribution f ~ v^2 exp(-v^2/vth^2): mean = 2 vth / sqrt(pi)
    assert s.mean() == pytest.approx(2 * 1000.0 / np.sqrt(np.pi), rel=1e-2)


def test_bird_gamma():
    import math
    for x in (0.5, 1.0, 1.5, 1.69, 2.5, 3.3):
        assert O.bird_gamma(x) == pytest.approx(math.gamma(x), rel=2e-4)


def _omesh(spec):
    return O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)


def test_node_volumes_cover_domain():
    spec = W.es_pic_mesh(21, 11, 1e-3)
    vol = O.node_volumes(_omesh(spec))
    Lx, Ly = spec.lengths()
    assert vol.sum() == pytest.approx(Lx * Ly, rel=1e-12)


def test_operator_structure_xy():
    """The FVM assembly reduces to the 5-point Laplacian inside, identity on Dirichlet
    nodes, central differences for the gradient (Solver.java:451-611)."""
    spec = W.es_pic_mesh(15, 9, 1e-3, electrode_halfwidth=1.5e-3)
    op = O.assemble(_omesh(spec))
    p, c, v = op["A"]
    ni = spec.ni
    dx = spec.dh[0]
    for j in range(1, spec.nj - 1):
        for i in range(1, ni - 1):
            u = j * ni + i
            row = dict(zip(c[p[u]:p[u + 1]], v[p[u]:p[u + 1]]))
            if op["fixed"][u]:
                assert row == {u: 1.0}
                continue
            assert set(row) == {u, u - 1, u + 1, u - ni, u + ni}
            assert row[u] * dx * dx == pytest.approx(-4.0, rel=1e-12)
            for k in (u - 1, u + 1, u - ni, u + ni):
                assert row[k] * dx * dx == pytest.approx(1.0, rel=1e-12)


def test_poisson_linear_limit_matches_laplace():
    """With a negligible electron density the NR solve is Laplace's equation; between
    phi = 1 on the left wall and 0 on the right with Neumann top/bottom the solution is linear."""
    ni, nj, dh = 17, 9, 1e-3
    nmax = max(ni, nj)
    node_type = np.full((nj, ni), O.NODE_OPEN, np.int8)
    node_type[:, 0] = node_type[:, -1] = O.NODE_DIRICHLET
    face = np.zeros((4, nmax), np.int8)
    face[O.F_TOP, :] = O.DB_SYMMETRY
    face[O.F_BOTTOM, :] = O.DB_SYMMETRY
    bc = np.zeros((nj, ni))
    bc[:, 0] = 1.0
    m = O.OMesh(ni, nj, [0, 0], [dh, dh], O.DOM_XY, node_type.reshape(-1), face)
    phi0 = np.zeros(ni * nj)
    phi, it, out = O.poisson_nl(m, bc.reshape(-1), np.zeros(ni * nj), 1e-20, 2.0, 0.0, 8.85418782e-12,
                                phi0, max_it=20000, tol=1e-12, nl_max_it=50, nl_tol=1e-10)
    exact = np.tile(1.0 - np.arange(ni) / (ni - 1), nj)
    assert np.max(np.abs(phi - exact)) < 1e-6


def test_push_ballistic_uniform_field():
    """No surfaces, uniform E: one push moves x by (v + qE/m dt) dt exactly."""
    spec = W.es_pic_mesh(41, 21, 1e-3, walls=O.DB_OPEN, electrode_halfwidth=1e-4)
    spec.seg_xy = np.zeros((0, 4))
    m = _omesh(spec)
    n = 100
    rng = np.random.default_rng(0)
    parts = np.zeros((n, 12))
    lc = np.column_stack([rng.uniform(10, 30, n), rng.uniform(5, 15, n)])
    parts[:, 6:8] = lc
    parts[:, 0:2] = lc * 1e-3
    parts[:, 3] = 50.0
    parts[:, 4] = -20.0
    parts[:, 9] = 1.0
    parts[:, 10] = 1
    E = 1000.0
    efi = np.full(spec.nn, E)
    efj = np.zeros(spec.nn)
    q, mass, dt = 1.6e-19, 1.6e-26, 1e-6
    alive, stats, _, _ = O.push(m, efi, efj, q, mass, dt, np.zeros((0, 9)), np.zeros(spec.nn + 1),
                                np.zeros(0), parts)
    assert alive == n
    vx = 50.0 + q / mass * E * dt
    assert np.allclose(parts[:, 3], vx, rtol=1e-14)
    assert np.allclose(parts[:, 6], lc[:, 0] + vx * dt / 1e-3, rtol=0, atol=1e-10)
    assert np.allclose(parts[:, 7], lc[:, 1] - 20.0 * dt / 1e-3, rtol=0, atol=1e-10)
    assert stats[0] == pytest.approx(n)


def test_scatter_conserves_weight():
    spec = W.es_pic_mesh(21, 11, 1e-3)
    m = _omesh(spec)
    vol = O.node_volumes(m)
    rng = np.random.default_rng(1)
    n = 1000
    parts = np.zeros((n, 12))
    parts[:, 6] = rng.uniform(0, 19.999, n)
    parts[:, 7] = rng.uniform(0, 9.999, n)
    parts[:, 9] = 3.0
    parts[:, 10] = 1
    den = O.update_fields(m, vol, parts)
    assert (den * vol).sum() == pytest.approx(3.0 * n, rel=1e-12)


def test_node_segments_box_rule():
    spec = W.es_pic_mesh(81, 41, 1e-3)
    ptr, idx = O.node_segments(_omesh(spec), spec.seg_xy)
    # every listed node lies within 2 cells of the electrode square
    ni = spec.ni
    nodes = np.repeat(np.arange(spec.nn), np.diff(ptr))
    i, j = nodes % ni, nodes // ni
    xlo, xhi = spec.seg_xy[:, 0].min() / 1e-3, spec.seg_xy[:, 0].max() / 1e-3
    assert i.min() >= np.floor(xlo) - 2 and i.max() <= np.ceil(xhi) + 2
    assert len(idx) > 0


# ---- the oracle reproduces its committed golden fixtures -------------------------------
import os  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_golden_java_random():
    g = np.load(os.path.join(GOLDEN, "java_random.npz"))
    assert np.array_equal(O.jrandom_doubles(0, 16), g["seed0"])
    assert np.array_equal(O.jrandom_doubles(42, 16), g["seed42"])
    assert np.array_equal(O.sample_maxw3d(7, 64, 1000.0), g["maxw3d_seed7"])


def test_golden_push():
    g = np.load(os.path.join(GOLDEN, "push_es_pic_81x41.npz"))
    spec = W.es_pic_mesh(81, 41, 1e-3)
    ion = W.IonSpecies()
    m = _omesh(spec)
    ptr, idx = O.node_segments(m, spec.seg_xy)
    lc, vel = g["lc0"], g["vel0"]
    P = np.zeros((lc.shape[0], 12))
    P[:, 0:2] = lc * np.array(spec.dh)
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = ion.spwt
    P[:, 10] = 1
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_ABSORB)
    O.push(m, g["efi"], g["efj"], ion.charge, ion.mass, float(g["dt"]), segs, ptr, idx, P)
    assert np.array_equal(P[:, 10].astype(np.int8), g["alive"])
    assert np.array_equal(P[:, 6:8], g["lc1"])
    assert np.array_equal(O.update_fields(m, O.node_volumes(m), P), g["den"])


def test_golden_poisson_residual_and_field():
    """The fixture potential satisfies the oracle operator at its FP64 floor, and its
    field / electron density are reproduced."""
    g = np.load(os.path.join(GOLDEN, "poisson_es_pic_81x41.npz"))
    spec = W.es_pic_mesh(81, 41, 1e-3)
    m = _omesh(spec)
    r = O.poisson_residual(m, spec.bc_value, g["rho"], 1e12, 2.0, 0.0, 8.85418782e-12, g["phi"])
    assert r / spec.nn < 1e-9
    efi, efj = O.efield(m, g["phi"])
    assert np.array_equal(efi, g["efi"]) and np.array_equal(efj, g["efj"])
    assert np.array_equal(O.boltzmann(g["phi"], 1e12, 2.0, 0.0), g["ne"])


def test_oracle_samples_known_answers():
    """updateSamples / computeFields: one particle scatters its weight bilinearly, has
    zero spread (T = 0 where sampled, T_init elsewhere) and counts once in its cell; a
    Maxwellian sample gives back its temperature."""
    spec = W.es_pic_mesh(11, 11, 1e-3)
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    P = np.zeros((1, 12))
    P[0, 6:8] = (2.25, 3.5)
    P[0, 3:6] = (100.0, -50.0, 10.0)
    P[0, 9] = 2.0
    P[0, 10] = 1
    sums = O.update_samples(m, P)
    sums = O.update_samples(m, P, sums)   # two samples of the same state
    ni = spec.ni
    c = sums[0].reshape(spec.nj, ni)
    assert c[3, 2] == pytest.approx(2 * 2.0 * 0.75 * 0.5)
    assert c[3, 3] == pytest.approx(2 * 2.0 * 0.25 * 0.5)
    assert c[4, 3] == pytest.approx(2 * 2.0 * 0.25 * 0.5)
    assert c[4, 2] == pytest.approx(2 * 2.0 * 0.75 * 0.5)
    assert sums[7].reshape(spec.nj, ni)[3, 2] == 2 and sums[7].sum() == 2
    vol = O.node_volumes(m)
    f = O.compute_fields(sums, 2, vol, 16 * 1.66053886e-27, 300.0)
    sampled = sums[0] > 0
    assert np.allclose(f["T"][sampled], 0.0, atol=1e-9)
    assert np.all(f["T"][~sampled] == 300.0)
    assert np.allclose(f["u-ave"][sampled], 100.0) and np.allclose(f["v-ave"][sampled], -50.0)
    assert f["mpc"].reshape(spec.nj, ni)[3, 2] == 1.0
    assert np.allclose(f["nd-ave"], sums[0] / 2 / vol)
    # Maxwellian at 500 K: T from the sampled second moments
    rng = np.random.default_rng(5)
    n = 200_000
    mass = 16 * 1.66053886e-27
    Q = np.zeros((n, 12))
    Q[:, 6] = rng.uniform(1, 9, n)
    Q[:, 7] = rng.uniform(1, 9, n)
    Q[:, 3:6] = rng.normal(0, np.sqrt(1.3806503e-23 * 500 / mass), (n, 3)) + [700.0, 0, 0]
    Q[:, 9] = 1.0
    Q[:, 10] = 1
    g = O.compute_fields(O.update_samples(m, Q), 1, vol, mass, 300.0)
    inner = (np.arange(spec.nj)[:, None] >= 2) & (np.arange(spec.nj)[:, None] <= 8) & \
            (np.arange(ni)[None, :] >= 2) & (np.arange(ni)[None, :] <= 8)
    assert np.mean(g["T"].reshape(spec.nj, ni)[inner]) == pytest.approx(500.0, rel=0.02)
    assert np.mean(g["u-ave"].reshape(spec.nj, ni)[inner]) == pytest.approx(700.0, rel=0.02)


def test_oracle_axisymmetric_source_area_weighted():
    """Spline.randomT on an axisymmetric mesh: positions uniform in the swept area, so on a
    radial inlet r in [0, R] the radius has density 2 r / R^2 (mean 2R/3, median R/sqrt 2),
    and the flux uses the frustum area pi (r1 + r2) L."""
    R = 5e-3
    seg = np.array([0.0, R, 0.0, 0.0])
    mass = 40 * 1.66053886e-27
    parts, _ = O.maxwellian_source(7, seg, 1e22, 500.0, 300.0, mass, 1e9, 1e-6, cap=1 << 20,
                                   domain=2)
    r = parts[:, 1]
    assert parts.shape[0] > 100_000
    assert np.mean(r) == pytest.approx(2 * R / 3, rel=5e-3)
    assert np.median(r) == pytest.approx(R / np.sqrt(2), rel=5e-3)
    # expected count from the frustum area (here a disc of radius R)
    v_mean = np.sqrt(8 * 1.3806503e-23 * 300.0 / (np.pi * mass))
    expect = 1e22 * np.pi * R * R * (500.0 + v_mean / 4) * 1e-6 / 1e9
    assert parts.shape[0] == int(expect)


def _ionization_case(n=4000, seed=5, eV=50.0):
    """Electrons of one energy, isotropic, uniform in a 21x21 XY box; a neutral target."""
    spec = W.es_pic_mesh(21, 21, 1e-3, walls=abi.DB_SYMMETRY, electrode_halfwidth=1e-12)
    spec.node_type[:] = abi.NODE_OPEN
    me = 9.10938e-31
    rng = np.random.default_rng(seed)
    lc = rng.uniform(0.5, 19.5, (n, 2))  # control volumes of full size
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    vel = d * np.sqrt(2 * eV * 1.60217646e-19 / me)
    P = np.zeros((n, 12))
    P[:, 0:2] = spec.x0 + lc * spec.dh
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = 2.5e6
    P[:, 10] = 1
    return spec, me, P


def test_oracle_mcc_ionization_known_answers():
    """ModelIonization (MCC.java:304-356) in the oracle: with a dense target every electron
    collides; each collided electron makes one more electron of the same speed (the
    reference's speed2a), keeps at most e - e_ion, and (int)(2.5 + rnd) ions are made per
    collision; delta_n, count_sum and real_sum add up exactly; S holds the energy term."""
    spec, me, P = _ionization_case()
    m = _omesh(spec)
    nn = spec.nn
    z = np.zeros(nn)
    den, T = np.full(nn, 1e26), np.full(nn, 300.0)
    e_ion, mi, spwt_i = 15.76, 40 * 1.66053886e-27, 1e6
    e0 = 0.5 * me * (P[:, 3:6] ** 2).sum(1) / 1.60217646e-19
    v0 = P[:, 3:6].copy()
    out = O.mcc_ex(m, P, me, mi, den, z, z, z, T, 1e-20, 5e-8, 2, 7, src_spwt=2.5e6, e_ion=e_ion,
                   prod_mass=mi, prod_spwt=spwt_i, max_new=20000)
    n = P.shape[0]
    assert out["cols"] == n and out["n_new_e"] == n
    e1 = 0.5 * me * (P[:, 3:6] ** 2).sum(1) / 1.60217646e-19
    assert np.all(e1 <= e0 - e_ion + 1e-9)
    assert abs(e1.mean() / ((e0 - e_ion).mean() / 2) - 1) < 0.05
    s_src = np.linalg.norm(P[:, 3:6], axis=1)
    s_new = np.linalg.norm(out["new_e"][:, 3:6], axis=1)
    assert np.allclose(s_new, s_src, rtol=1e-12)
    assert np.array_equal(out["new_e"][:, 6:8], P[:, 6:8])
    ratio = out["n_new_i"] / out["cols"]
    assert 2.4 < ratio < 2.6
    assert out["delta_n"].sum() == pytest.approx(spwt_i * out["n_new_i"], rel=1e-12)
    assert out["count_sum"].sum() == out["cols"]
    assert out["real_sum"].sum() == pytest.approx(2.5e6 * out["cols"], rel=1e-12)
    # interior particles only touch nodes with the full control volume dx*dy (XY depth 1):
    # the scattered S sums to sum mpw (E1 - E2) / (dt dx dy) with E = 0.5 m |v|
    interior = np.all((P[:, 6:8] >= 0.5) & (P[:, 6:8] <= 19.5), axis=1)
    assert interior.all()
    dE = 0.5 * me * (np.linalg.norm(v0, axis=1) - s_src)
    assert out["S"].sum() == pytest.approx((2.5e6 * dE / (5e-8 * 1e-6)).sum(), rel=1e-9)
    # ions: Maxwellian at 300 K with the sampler's 1.2 factor
    vi = out["new_i"][:, 3:6]
    sig = 1.2 * np.sqrt(2 * 1.3806503e-23 * 300 / mi) / np.sqrt(2)
    assert abs(vi.std() / sig - 1) < 0.05


def test_oracle_mcc_ex_matches_plain_for_mex_cex():
    """The extended entry point draws the same random numbers for MEX and CEX."""
    spec, me, P = _ionization_case(n=2000, seed=9)
    m = _omesh(spec)
    nn = spec.nn
    z = np.zeros(nn)
    den, T = np.full(nn, 1e20), np.full(nn, 300.0)
    for model in (0, 1):
        A, B = P.copy(), P.copy()
        ca = O.mcc(m, A, me, 40 * 1.66e-27, den, z, z, z, T, 1e-20, 5e-8, model, 3)
        out = O.mcc_ex(m, B, me, 40 * 1.66e-27, den, z, z, z, T, 1e-20, 5e-8, model, 3)
        assert ca == out["cols"] > 0
        assert np.array_equal(A, B)


def test_oracle_point_internal_electrode_box():
    """BoundaryModule.isInternal on the 9x9 mm electrode box of the ES-PIC mesh: inside,
    on an edge and outside points."""
    spec = W.es_pic_mesh(81, 41, 1e-3)
    seg, bt = spec.seg_xy, spec.seg_btype
    assert O.point_internal(seg, bt, 0.040, 0.020)          # centre
    assert O.point_internal(seg, bt, 0.0440, 0.0199)        # inside, near the right side
    assert O.point_internal(seg, bt, 0.0445, 0.020)         # on the right side
    assert not O.point_internal(seg, bt, 0.0450, 0.020)     # just outside
    assert not O.point_internal(seg, bt, 0.005, 0.035)      # far away


def test_oracle_preload_and_uniform_source_known_answers():
    """VolumePreloadSource: ceil(den V / spwt) - 1 particles per cell, none inside the
    electrode, Maxwellian with the 1.2 factor.  UniformSource: the Source.regenerate count
    and v = normal * v_drift."""
    spec = W.es_pic_mesh(41, 21, 1e-3)
    mass, spwt, den, T, dt = 16 * 1.66053886e-27, 1e3, 1e12, 1000.0, 5e-7
    parts = O.preload(3, spec, den, T, mass, spwt, dt)
    per_cell = int(np.ceil(den * 1e-6 / spwt)) - 1
    total = per_cell * 40 * 20
    inside_frac = (9e-3 * 9e-3) / (40e-3 * 20e-3)
    assert abs(parts.shape[0] - total * (1 - inside_frac)) < 6 * np.sqrt(total * inside_frac)
    assert not any(O.point_internal(spec.seg_xy, spec.seg_btype, x, y) for x, y in parts[:2000, 0:2])
    sig = 1.2 * np.sqrt(2 * 1.3806503e-23 * T / mass) / np.sqrt(2)
    assert abs(parts[:, 3:6].std() / sig - 1) < 0.02
    seg = np.array([0.0, 0.02, 0.0, 0.0])  # normal (-dy, dx)/L = (1, 0)
    mdot, v = 1e-12, 5000.0
    p1, rem = O.uniform_source(4, seg, mdot, v, mass, spwt, dt)
    expect = mdot * dt / (mass * spwt)
    assert p1.shape[0] == int(expect) and rem == pytest.approx(expect - int(expect))
    assert np.all(p1[:, 3] == v) and np.all(p1[:, 4] == 0) and np.all(p1[:, 5] == 0)
    assert np.all((p1[:, 1] >= 0) & (p1[:, 1] <= 0.02))


def test_oracle_dsmc_collision_rate_matches_vhs_theory():
    """NTC with the Bird 4.63 VHS cross-section in one cell of an equilibrium gas: the
    expected collisions per step are N^2 w dt <sigma g> / (2 V), where for a Maxwellian
    relative speed at temperature T
        <sigma g> = sigma0 (2 k T_ref / m_r)^(omega - 1/2) (2 k T / m_r)^(1 - omega) / Gamma(3/2)
    (at T = T_ref this is sigma0 times the mean relative speed).  Elastic collisions keep
    momentum and energy."""
    import math
    KB, mass, d, T_ref, om = 1.3806503e-23, 6.63e-26, 4.17e-10, 273.0, 0.81
    mr = 0.5 * mass
    sigma0 = math.pi * d * d
    V, dt, n = 1e-9, 1e-6, 2000
    for T, seed in ((273.0, 3), (819.0, 4)):
        rng = np.random.default_rng(seed)
        P = np.zeros((n, 12))
        P[:, 3:6] = rng.normal(0.0, math.sqrt(KB * T / mass), (n, 3))
        P[:, 6:8] = 0.5
        P[:, 10] = 1
        sg = sigma0 * (2 * KB * T_ref / mr) ** (om - 0.5) * (2 * KB * T / mr) ** (1 - om) / math.gamma(1.5)
        spwt = 2e4 * 2 * V / (n * n * dt * sg)  # about 2e4 collisions expected
        P[:, 9] = spwt
        state = np.array([[6.0 * sg, 0.0]])  # (sigma g)_max well above every pair's sigma g
        counts = np.zeros((1, 2))
        p0, e0 = P[:, 3:6].sum(axis=0), (P[:, 3:6] ** 2).sum()
        # the pair average over this finite sample differs from the Maxwellian one by
        # about 1 %, the count by its Poisson spread (0.7 %)
        got = O.dsmc(2, 2, np.array([V]), P, mass, spwt, d, T_ref, om, 1.0, dt, state, counts, seed)
        assert got == pytest.approx(2e4, rel=0.04)
        assert counts[0, 0] == got
        assert np.allclose(P[:, 3:6].sum(axis=0), p0, atol=1e-9 * np.abs(P[:, 3:6]).sum())
        assert (P[:, 3:6] ** 2).sum() == pytest.approx(e0, rel=1e-12)


def test_oracle_dsmc_pair_rate_and_boyd_update():
    """Two materials (argon and helium) in one equilibrium cell.  With equal weights the NTC
    count of an unlike pair is N1 N2 w dt <sigma g> / V (nsel doubled for two species,
    denominator Pab + Pba = 2), with <sigma g> for the reduced mass and the pair's mean
    d, T_ref and omega (SigmaBird463.init), and elastic collisions keep the mass-weighted
    momentum and the kinetic energy.  With weights w2 = w1 / 4 the count follows the
    reference's expression 2 (N1 w1 / V) N2 dt <sigma g> / (Pab + (w2/w1) Pba) with Pab = 1/4,
    Pba = 1 (DSMC.java:276-290; for unequal weights this is w1/w2 times N1 N2 w1 dt <sigma g>
    / V, and parity keeps it), and a collision moves particle 1 with probability w2/w1 and
    particle 2 always (Boyd's update, :431-452)."""
    import math
    KB, AMU = 1.3806503e-23, 1.66053886e-27
    m1, m2 = 40 * AMU, 4 * AMU
    mat1 = dict(diam=4.17e-10, T_ref=273.0, omega=0.81, vss_alpha=1.0)
    mat2 = dict(diam=2.33e-10, T_ref=273.0, omega=0.66, vss_alpha=1.0)
    mr = m1 * m2 / (m1 + m2)
    d = 0.5 * (mat1["diam"] + mat2["diam"])
    om = 0.5 * (mat1["omega"] + mat2["omega"])
    T_ref = 273.0
    V, dt, n1, n2, T = 1e-9, 1e-6, 1500, 1000, 500.0
    sg = math.pi * d * d * (2 * KB * T_ref / mr) ** (om - 0.5) * (2 * KB * T / mr) ** (1 - om) / math.gamma(1.5)
    for ratio, seed in ((1.0, 5), (0.25, 6)):
        rng = np.random.default_rng(seed)
        P1 = np.zeros((n1, 12))
        P2 = np.zeros((n2, 12))
        P1[:, 3:6] = rng.normal(0.0, math.sqrt(KB * T / m1), (n1, 3))
        P2[:, 3:6] = rng.normal(0.0, math.sqrt(KB * T / m2), (n2, 3))
        P1[:, 6:8] = P2[:, 6:8] = 0.5
        P1[:, 10] = P2[:, 10] = 1
        den = ratio + ratio * 1.0  # Pab + (w2/w1) Pba
        w1 = 2e4 * V * den / (2 * n1 * n2 * dt * sg)  # about 2e4 collisions expected
        w2 = w1 * ratio
        P1[:, 9], P2[:, 9] = w1, w2
        state = np.array([[6.0 * sg, 0.0]])
        counts = np.zeros((1, 2))
        v1, v2 = P1[:, 3:6].copy(), P2[:, 3:6].copy()
        p0 = m1 * v1.sum(axis=0) + m2 * v2.sum(axis=0)
        e0 = m1 * (v1 ** 2).sum() + m2 * (v2 ** 2).sum()
        got = O.dsmc_pair(2, 2, np.array([V]), P1, m1, w1, P2, m2, w2, mat1, mat2, dt, state, counts, seed)
        assert got == pytest.approx(2e4, rel=0.05)
        assert counts[0, 0] == got
        assert counts[0, 1] == pytest.approx(got * 0.5 * (w1 + w2), rel=1e-12)
        moved1 = np.any(P1[:, 3:6] != v1, axis=1).sum()
        moved2 = np.any(P2[:, 3:6] != v2, axis=1).sum()
        if ratio == 1.0:
            p1 = m1 * P1[:, 3:6].sum(axis=0) + m2 * P2[:, 3:6].sum(axis=0)
            e1 = m1 * (P1[:, 3:6] ** 2).sum() + m2 * (P2[:, 3:6] ** 2).sum()
            assert np.allclose(p1, p0, atol=1e-9 * (m1 * np.abs(v1).sum()))
            assert e1 == pytest.approx(e0, rel=1e-12)
        else:
            # each collision moves particle 2, and particle 1 with probability 1/4: among
            # 1500 argon and 1000 helium particles, nearly every helium particle and
            # about 1 - exp(-got / 4 / n1) of the argon particles have moved
            assert moved2 > 0.99 * n2
            f1 = 1 - math.exp(-got * 0.25 / n1)
            assert abs(moved1 / n1 - f1) < 0.05


def test_oracle_poisson_boltzmann_debye_shielding():
    """Boltzmann electrons over a uniform ion background e n0, walls at phi_w << kTe on the
    left and right, Neumann top and bottom: the linearised equation phi'' = phi / lambda_D^2
    (lambda_D^2 = eps kTe / (e n0)) has on the grid the exact solution
        phi_i = phi_w cosh(kappa (i - N/2)) / cosh(kappa N / 2),  cosh kappa = 1 + h^2 / (2 lambda_D^2).
    The nonlinear solve must agree to the size of the neglected term, (phi / kTe) / 2."""
    import math
    QE, EPS = 1.602176565e-19, 8.85418782e-12
    n0, kTe, phi_w = 1e12, 2.0, 0.01
    lam = math.sqrt(EPS * kTe / (QE * n0))
    ni, nj, h = 65, 5, lam / 8
    node_type = np.full((nj, ni), O.NODE_OPEN, np.int8)
    node_type[:, 0] = node_type[:, -1] = O.NODE_DIRICHLET
    face = np.zeros((4, ni), np.int8)
    face[O.F_TOP, :] = O.DB_SYMMETRY
    face[O.F_BOTTOM, :] = O.DB_SYMMETRY
    bc = np.zeros((nj, ni))
    bc[:, 0] = bc[:, -1] = phi_w
    m = O.OMesh(ni, nj, [0, 0], [h, h], O.DOM_XY, node_type.reshape(-1), face)
    phi, it, out = O.poisson_nl(m, bc.reshape(-1), np.full(ni * nj, QE * n0), n0, kTe, 0.0, EPS,
                                np.zeros(ni * nj), max_it=200000, tol=1e-13, nl_max_it=100, nl_tol=1e-12)
    kap = math.acosh(1 + h * h / (2 * lam * lam))
    i = np.arange(ni)
    exact = phi_w * np.cosh(kap * (i - (ni - 1) / 2)) / np.cosh(kap * (ni - 1) / 2)
    assert np.max(np.abs(phi.reshape(nj, ni) - exact[None, :])) < 0.5 * phi_w / kTe * phi_w
    assert phi.reshape(nj, ni)[2, ni // 2] < 0.05 * phi_w  # shielded over 4 Debye lengths


@pytest.mark.parametrize("domain", [O.DOM_ZR, O.DOM_RZ])
def test_oracle_axisymmetric_rotation_known_answer(domain):
    """A particle with only a theta velocity w at radius r0 (no field): after dt its radius is
    sqrt(r0^2 + (w dt)^2), its velocity turns by alpha = atan(w dt / r0) into the radial
    direction (v_r = w sin alpha, v_theta = w cos alpha) and theta advances by alpha
    (rotateToZR / rotateToRZ, KineticMaterial.java:424-462)."""
    ni, nj, dh = 41, 41, 1e-3
    rad = 1 if domain == O.DOM_ZR else 0  # the radial coordinate: y in ZR, x in RZ
    x0 = [0.0, 0.0]
    x0[rad] = 0.01
    node_type = np.full(ni * nj, O.NODE_OPEN, np.int8)
    face = np.full((4, ni), O.DB_OPEN, np.int8)
    m = O.OMesh(ni, nj, x0, [dh, dh], domain, node_type, face)
    w, dt = 3000.0, 1e-6
    r0 = np.array([0.012, 0.02, 0.03])
    parts = np.zeros((3, 12))
    parts[:, 1 - rad] = 0.02
    parts[:, rad] = r0
    parts[:, 6 + (1 - rad)] = 0.02 / dh
    parts[:, 6 + rad] = (r0 - 0.01) / dh
    parts[:, 5] = w
    parts[:, 9] = 1.0
    parts[:, 10] = 1
    zero = np.zeros(ni * nj)
    alive, _, _, _ = O.push(m, zero, zero, 1.6e-19, 6.6e-26, dt, np.zeros((0, 9)), np.zeros(ni * nj + 1),
                            np.zeros(0), parts)
    assert alive == 3
    R = np.hypot(r0, w * dt)
    assert np.allclose(parts[:, rad], R, rtol=1e-14)
    assert np.allclose(parts[:, 3 + rad], w * (w * dt) / R, rtol=1e-12)
    assert np.allclose(parts[:, 5], w * r0 / R, rtol=1e-12)
    assert np.allclose(parts[:, 1 - rad], 0.02, rtol=1e-15)
    assert np.allclose(np.abs(parts[:, 2]), np.arctan2(w * dt, r0), rtol=1e-12)
    assert np.allclose(parts[:, 6 + rad], (R - 0.01) / dh, rtol=1e-12)


@pytest.mark.parametrize("domain", [O.DOM_ZR, O.DOM_RZ])
def test_oracle_ruyten_scatter_uniform_density(domain):
    """Particles uniform in volume over a cylinder from the axis (radius drawn as
    R sqrt(U)): with Ruyten's radial weights (Field2D.java:254-285) and the annular node
    volumes the density comes out uniform on every radial row, the axis row and the outer
    row included, and the deposited weight is conserved exactly."""
    ni = nj = 21
    dh = 1e-3
    rad = 1 if domain == O.DOM_ZR else 0
    node_type = np.full(ni * nj, O.NODE_OPEN, np.int8)
    face = np.full((4, ni), O.DB_OPEN, np.int8)
    m = O.OMesh(ni, nj, [0.0, 0.0], [dh, dh], domain, node_type, face)
    vol = O.node_volumes(m)
    rng = np.random.default_rng(2)
    n = 2_000_000
    L = (ni - 1) * dh
    parts = np.zeros((n, 12))
    parts[:, 6 + rad] = np.sqrt(rng.uniform(0, 1, n)) * L / dh
    parts[:, 6 + (1 - rad)] = rng.uniform(0, L, n) / dh
    parts[:, 9] = 1.0
    parts[:, 10] = 1
    den = O.update_fields(m, vol, parts)
    assert (den * vol).sum() == pytest.approx(n, rel=1e-12)
    d = (den * np.pi * L * L * L / n).reshape(nj, ni)
    v = vol.reshape(nj, ni)
    if rad == 0:  # radius along i: radial rows are columns
        d, v = d.T, v.T
    # mean over the interior axial positions of each radial row, against its Poisson spread
    mean = d[:, 1:-1].mean(axis=1)
    spread = 1 / np.sqrt(n * v[:, ni // 2] / (np.pi * L ** 3) * (ni - 2))
    assert np.all(np.abs(mean - 1) < 4 * spread), (mean, spread)


@pytest.mark.parametrize("domain", [O.DOM_XY, O.DOM_ZR, O.DOM_RZ])
def test_oracle_efield_of_linear_potential(domain):
    """E = -grad(phi) (Solver.evaluateGradient, Solver.java:789-814) is exact for a linear
    potential on every node, the one-sided edge differences included."""
    ni, nj, dx, dy = 17, 9, 2e-3, 1e-3
    node_type = np.full(ni * nj, O.NODE_OPEN, np.int8)
    face = np.full((4, ni), O.DB_DIRICHLET, np.int8)
    m = O.OMesh(ni, nj, [0.0, 0.005], [dx, dy], domain, node_type, face)
    i, j = np.meshgrid(np.arange(ni), np.arange(nj))
    phi = (3.0 + 120.0 * i * dx - 45.0 * (0.005 + j * dy)).reshape(-1)
    efi, efj = O.efield(m, phi)
    assert np.allclose(efi, -120.0, rtol=0, atol=1e-9)
    assert np.allclose(efj, 45.0, rtol=0, atol=1e-9)


def test_oracle_mcc_cex_rate_known_answer():
    """MCC.perform with CEX (MCC.java:167-221, 287-297) against a cold uniform target: each
    ion of speed g collides with probability 1 - exp(-n sigma g dt) and then moves with the
    target's (near-zero) velocity."""
    spec = W.es_pic_mesh(21, 21, 1e-3, walls=abi.DB_SYMMETRY, electrode_halfwidth=1e-12)
    spec.node_type[:] = abi.NODE_OPEN
    m = _omesh(spec)
    nn, n = spec.nn, 200_000
    mi = 40 * 1.66053886e-27
    rng = np.random.default_rng(4)
    lc = rng.uniform(0.5, 19.5, (n, 2))
    P = np.zeros((n, 12))
    P[:, 0:2] = spec.x0 + lc * spec.dh
    P[:, 6:8] = lc
    P[:, 3] = 1e4
    P[:, 9] = 1.0
    P[:, 10] = 1
    z = np.zeros(nn)
    sigma, dt, tden = 1e-19, 1e-6, 1e20
    cols = O.mcc(m, P, mi, mi, np.full(nn, tden), z, z, z, np.full(nn, 1e-3), sigma, dt, 1, 11)
    p = 1 - np.exp(-tden * sigma * 1e4 * dt)
    assert abs(cols - n * p) < 4 * np.sqrt(n * p * (1 - p))
    assert (np.linalg.norm(P[:, 3:6], axis=1) < 10.0).sum() == cols  # target thermal speed ~1 m/s


def test_oracle_specular_reflection_known_answer():
    """Ions moving +x into the electrode box's left face (outward normal -x) with the specular
    handler (SurfaceInteraction.java:104-125): the velocity becomes v + n sqrt(2) |v_xy|,
    at normal incidence (1 - sqrt(2)) v; they stay on the gas side and keep their y."""
    spec = W.es_pic_mesh(81, 41, 1e-3)  # box x in [35.5, 44.5] mm, y in [15.5, 24.5] mm
    m = _omesh(spec)
    ptr, idx = O.node_segments(m, spec.seg_xy)
    rng = np.random.default_rng(8)
    n = 2000
    lc = np.column_stack([rng.uniform(33.0, 35.0, n), rng.uniform(17.0, 23.0, n)])
    P = np.zeros((n, 12))
    P[:, 0:2] = lc * 1e-3
    P[:, 3] = 8000.0
    P[:, 6:8] = lc
    P[:, 9] = 1e6
    P[:, 10] = 1
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_SPECULAR)
    zero = np.zeros(spec.nn)
    alive, _, _, _ = O.push(m, zero, zero, 1.602e-19, 16 * 1.66053886e-27, 5e-7, segs, ptr, idx, P)
    assert alive == n
    assert np.allclose(P[:, 3], 8000.0 * (1 - np.sqrt(2.0)), rtol=1e-12)
    assert np.all(P[:, 4] == 0.0) and np.all(P[:, 5] == 0.0)
    assert np.all(P[:, 0] < 0.0355) and np.allclose(P[:, 1], lc[:, 1] * 1e-3, rtol=0, atol=1e-15)


def test_oracle_diffuse_reflection_cosine_law():
    """The diffuse handler with full accommodation (SurfaceInteraction.java:127-213): speeds
    from the wall's Maxwellian speed distribution (mean 2/sqrt(pi) vth), directions by the
    cosine law about the outward normal (mean cosine 2/3), all away from the face."""
    spec = W.es_pic_mesh(81, 41, 1e-3)
    m = _omesh(spec)
    ptr, idx = O.node_segments(m, spec.seg_xy)
    rng = np.random.default_rng(9)
    n = 40000
    lc = np.column_stack([rng.uniform(33.0, 35.0, n), rng.uniform(17.0, 23.0, n)])
    P = np.zeros((n, 12))
    P[:, 0:2] = lc * 1e-3
    P[:, 3] = 8000.0
    P[:, 6:8] = lc
    P[:, 9] = 1e6
    P[:, 10] = 1
    mass = 16 * 1.66053886e-27
    vth = np.sqrt(2 * 1.3806503e-23 * 300.0 / mass)
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_DIFFUSE, vth=vth, c_rest=1.0, c_accom=1.0)
    zero = np.zeros(spec.nn)
    # a short step: the reflected particles cannot reach another face of the box
    alive, _, _, _ = O.push(m, zero, zero, 1.602e-19, mass, 5e-7, segs, ptr, idx, P)
    assert alive == n
    v = P[:, 3:6]
    speed = np.linalg.norm(v, axis=1)
    assert np.all(v[:, 0] <= 0)
    assert abs(speed.mean() / (2 / np.sqrt(np.pi) * vth) - 1) < 0.02
    assert abs((-v[:, 0] / speed).mean() - 2 / 3) < 0.01


def test_oracle_absorbed_flux_and_deposit_split():
    """A beam absorbed by the electrode box's left face (Material.java:759-796 through
    ProcessBoundary): every ion is removed; the face's two end values of the flux and the
    deposit hold its weight split linearly by the hit point's position along the face, so
    the two ends sum to N w and the far end holds w * sum(t)."""
    spec = W.es_pic_mesh(81, 41, 1e-3)
    m = _omesh(spec)
    ptr, idx = O.node_segments(m, spec.seg_xy)
    x1, y1, x2, y2 = spec.seg_xy[0]
    assert x1 == x2 and abs(x1 - 0.0355) < 1e-12  # the left face
    rng = np.random.default_rng(10)
    n, w = 3000, 2.5e5
    lc = np.column_stack([rng.uniform(33.0, 35.0, n), rng.uniform(16.0, 24.0, n)])
    P = np.zeros((n, 12))
    P[:, 0:2] = lc * 1e-3
    P[:, 3] = 8000.0
    P[:, 6:8] = lc
    P[:, 9] = w
    P[:, 10] = 1
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_ABSORB)
    zero = np.zeros(spec.nn)
    alive, _, flux, dep = O.push(m, zero, zero, 1.602e-19, 16 * 1.66053886e-27, 5e-7, segs, ptr, idx, P)
    assert alive == 0
    t = (lc[:, 1] * 1e-3 - y1) / (y2 - y1)
    for f in (flux, dep):
        assert f[0] + f[1] == pytest.approx(n * w, rel=1e-12)
        assert f[1] == pytest.approx(w * t.sum(), rel=1e-9)
        assert np.all(f[2:] == 0)


@pytest.mark.parametrize("domain", [O.DOM_ZR, O.DOM_RZ])
def test_oracle_axisymmetric_operator_on_quadratics(domain):
    """The FVM assembly on an axisymmetric mesh (Solver.java:451-553) is exact for quadratics
    at interior nodes, with the reference's scaling: face terms carry the face radius R and
    rows are divided by nodeVol = 2 pi area r (Mesh.java:998-1020), so A phi equals the
    cylindrical Laplacian over 2 pi: r^2 -> 4 / 2pi, z^2 -> 2 / 2pi."""
    ni = nj = 17
    dh = 1e-3
    rad = 1 if domain == O.DOM_ZR else 0
    node_type = np.full(ni * nj, O.NODE_OPEN, np.int8)
    face = np.full((4, ni), O.DB_DIRICHLET, np.int8)
    m = O.OMesh(ni, nj, [0.0, 0.0], [dh, dh], domain, node_type, face)
    p, c, v = O.assemble(m)["A"]
    i, j = np.meshgrid(np.arange(ni), np.arange(nj))
    r = (j if rad else i) * dh
    z = (i if rad else j) * dh
    for phi, lap in ((r ** 2, 4.0), (z ** 2, 2.0), (r ** 2 + 3 * z ** 2 + 5 * z, 10.0)):
        f = phi.reshape(-1)
        Af = np.array([np.dot(v[p[u]:p[u + 1]], f[c[p[u]:p[u + 1]]]) for u in range(ni * nj)]).reshape(nj, ni)
        assert np.allclose(Af[1:-1, 1:-1], lap / (2 * np.pi), rtol=1e-9)


def test_oracle_xy_maxwellian_source_known_answer():
    """MaxwellianSource on an XY inlet (MaxwellianSource.java:93-125, Source.java:167-198):
    the count per step is den L (v_drift + v_mean / 4) dt / w with the fraction carried;
    the velocity is the drift along the inward normal plus SampleMaxw3D (the sampler's 1.2
    spread factor, Utils.java:27-57); positions are uniform along the segment."""
    seg = np.array([0.0, 0.04, 0.0, 0.0])
    mass = 16 * 1.66053886e-27
    den, vd, T, spwt, dt = 1e12, 7000.0, 1000.0, 5e2, 5e-7
    parts, rem = O.maxwellian_source(7, seg, den, vd, T, mass, spwt, dt, cap=1 << 22, domain=0)
    v_mean = np.sqrt(8 * 1.3806503e-23 * T / (np.pi * mass))
    expect = den * 0.04 * (vd + v_mean / 4) * dt / spwt
    assert parts.shape[0] == int(expect) and rem == pytest.approx(expect - int(expect), abs=1e-6)
    sig = np.sqrt(1.3806503e-23 * T / mass)
    assert parts[:, 3].mean() == pytest.approx(vd, abs=6 * 1.2 * sig / np.sqrt(parts.shape[0]))
    assert parts[:, 4].std() == pytest.approx(1.2 * sig, rel=0.01)
    assert parts[:, 1].mean() == pytest.approx(0.02, abs=6 * 0.04 / np.sqrt(12 * parts.shape[0]))
    assert parts[:, 1].min() >= 0.0 and parts[:, 1].max() <= 0.04


@pytest.mark.parametrize("domain,x0", [(2, (0.0, 0.0)), (1, (0.0, 0.0)), (2, (0.0, 2e-3))])
def test_oracle_axisymmetric_rows_are_the_closed_form(domain, x0):
    """The device's closed-form axisymmetric operator: on a uniform RZ / ZR mesh every
    interior row of the reference's FVM assembly (Solver.java:451-553, face fluxes weighted
    by the face radius over the node volume 2 pi r dA, Mesh.java:998-1020) is
    [r c_a (axial neighbours) + c_r (r+ (radial up) + r- (radial down))] / (2 pi r), and the
    open-face rows are plain one-sided gradients."""
    from starfish_gb300 import abi
    ni, nj = 17, 9
    dh = (1e-3, 5e-4) if domain == abi.DOMAIN_ZR else (5e-4, 1e-3)
    nt = np.full(ni * nj, abi.NODE_OPEN, np.int8)
    face = np.full((4, max(ni, nj)), abi.DB_OPEN, np.int8)
    face[abi.FACE_BOTTOM if domain == abi.DOMAIN_ZR else abi.FACE_LEFT, :] = abi.DB_SYMMETRY
    nt[5 * ni + 8] = abi.NODE_DIRICHLET
    m = O.OMesh(ni, nj, x0, dh, domain, nt, face)
    ptr, col, val = O.assemble(m)["A"]
    cx, cy = 1 / dh[0] ** 2, 1 / dh[1] ** 2
    for j in range(nj):
        for i in range(ni):
            u = j * ni + i
            row = dict(zip(col[ptr[u]:ptr[u + 1]], val[ptr[u]:ptr[u + 1]]))
            if nt[u] == abi.NODE_DIRICHLET:
                assert row == {u: 1.0}
                continue
            if i in (0, ni - 1) or j in (0, nj - 1):
                # one-sided gradient rows (radius-free)
                h = dh[0] if i in (0, ni - 1) else dh[1]
                assert sorted(abs(v) for v in row.values()) == pytest.approx([1 / h, 1 / h], rel=1e-12)
                continue
            if domain == abi.DOMAIN_ZR:
                r = x0[1] + j * dh[1]
                exp = {u - 1: cx / (2 * np.pi), u + 1: cx / (2 * np.pi),
                       u + ni: cy * (r + dh[1] / 2) / (2 * np.pi * r), u - ni: cy * (r - dh[1] / 2) / (2 * np.pi * r)}
            else:
                r = x0[0] + i * dh[0]
                exp = {u + 1: cx * (r + dh[0] / 2) / (2 * np.pi * r), u - 1: cx * (r - dh[0] / 2) / (2 * np.pi * r),
                       u - ni: cy / (2 * np.pi), u + ni: cy / (2 * np.pi)}
            exp[u] = -sum(exp.values())
            for k, v in row.items():
                assert v == pytest.approx(exp.get(k, 0.0), rel=1e-12, abs=1e-9 * abs(exp[u]))
            for k, v in exp.items():
                assert row.get(k, 0.0) == pytest.approx(v, rel=1e-12)
