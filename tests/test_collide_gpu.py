"""DSMC and MCC on the GPU against the oracle (DSMC.java collideCell + ModelElastic,
MCC.java perform).  The random streams differ (Philox vs java.util.Random), so the
checks are statistical: collision counts, temperature relaxation and the conservation
laws of elastic collisions."""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

AMU = 1.66053886e-27
KB = 1.3806503e-23


def box_mesh(n=21, dh=1e-3):
    """XY box, all faces symmetry, no segments."""
    spec = W.es_pic_mesh(n, n, dh, walls=abi.DB_SYMMETRY, electrode_halfwidth=1e-12)
    spec.seg_xy = np.zeros((0, 4))
    spec.seg_btype = np.zeros(0, np.int32)
    spec.node_type[:] = abi.NODE_OPEN
    spec.bc_value[:] = 0
    return spec


def anisotropic_gas(spec, n, seed, Tx=600.0, Ty=150.0, Tz=150.0, mass=40 * AMU):
    rng = np.random.default_rng(seed)
    L = (spec.ni - 1)
    lc = rng.uniform(0, L, (n, 2))
    lc = np.floor(lc) + (lc - np.floor(lc)).astype(np.float32).astype(np.float64)
    sig = np.sqrt(KB * np.array([Tx, Ty, Tz]) / mass)
    vel = (rng.standard_normal((n, 3)) * sig).astype(np.float32).astype(np.float64)
    return lc, vel


def _om(spec):
    return O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)


def temps(vel, mass=40 * AMU):
    v = vel - vel.mean(axis=0)
    return mass * (v ** 2).mean(axis=0) / KB




def test_dsmc_relaxation_matches_oracle(gpulib):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, DSMC
    spec = box_mesh()
    mass, spwt, dt = 40 * AMU, 1e12, 1e-5
    n = 40000
    lc, vel = anisotropic_gas(spec, n, 1)
    # GPU
    dom = GpuDomain(spec)
    dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
    km = KineticMaterial(dom, mass, 0.0, spwt, capacity=n + 16)
    km.add_particles_lc(lc, vel)
    ds = DSMC(dom, km, model=abi.SIGMA_BIRD463, diam=4.17e-10, T_ref=273.0, omega=0.81)
    g_hist, g_cols = [], []
    for k in range(12):
        g_cols.append(ds.perform(dt))
        _, v = km.download()
        g_hist.append(temps(v))
    _, v_end = km.download()
    dom.close()
    # oracle
    P = np.zeros((n, 12))
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = spwt
    P[:, 10] = 1
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    cv = O.cell_volumes(m)
    nc = (spec.ni - 1) * (spec.nj - 1)
    state = np.zeros((nc, 2))
    state[:, 0] = 1e-16
    counts = np.zeros((nc, 2))
    o_hist, o_cols = [], []
    for k in range(12):
        o_cols.append(O.dsmc(spec.ni, spec.nj, cv, P, mass, spwt, 4.17e-10, 273.0, 0.81, 1.0, dt, state, counts, k))
        o_hist.append(temps(P[:, 3:6]))
    g_hist, o_hist = np.array(g_hist), np.array(o_hist)
    # collision counts per step agree statistically (after the sig_cr_max warm-up step)
    gc, oc = np.array(g_cols[2:], float), np.array(o_cols[2:], float)
    assert gc.mean() == pytest.approx(oc.mean(), rel=0.05)
    # the anisotropy relaxes at the same rate
    ga = g_hist[:, 0] - g_hist[:, 1]
    oa = o_hist[:, 0] - o_hist[:, 1]
    assert ga[-1] < 0.5 * ga[0]
    assert np.allclose(ga, oa, rtol=0.15, atol=15.0)
    # elastic collisions conserve momentum and energy (FP32 velocities)
    p0, p1 = vel.sum(axis=0), v_end.sum(axis=0)
    e0, e1 = (vel ** 2).sum(), (v_end ** 2).sum()
    assert np.all(np.abs(p1 - p0) <= 1e-4 * np.abs(vel).sum(axis=0))
    assert e1 == pytest.approx(e0, rel=1e-5)


def test_mcc_cex_collision_rate(gpulib):
    """Charge exchange of ions in a uniform neutral background: the number of collisions
    matches sum(1 - exp(-sigma g dt n)) (MCC.java:194-197) and the oracle."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, MCC
    spec = box_mesh()
    n = 200000
    mass = 40 * AMU
    lc, vel = anisotropic_gas(spec, n, 5, Tx=2e4, Ty=2e4, Tz=2e4)
    vel[:, 0] += 3000.0
    vel = vel.astype(np.float32).astype(np.float64)
    nn = spec.nn
    den = np.full(nn, 1e20)
    T = np.full(nn, 300.0)
    sigma, dt = 5e-19, 2e-6
    dom = GpuDomain(spec)
    dom.set_efield(np.zeros(nn), np.zeros(nn))
    km = KineticMaterial(dom, mass, 1.6e-19, 1.0, capacity=n + 16)
    km.add_particles_lc(lc, vel)
    mcc = MCC(dom, km, target_mass=mass, den=den, temp=T, model=abi.MCC_CEX, sigma_model=abi.SIGMA_CONST,
              c=[sigma, 0, 0, 0])
    cols = mcc.perform(dt)
    _, v_after = km.download()
    dom.close()
    g = np.linalg.norm(vel, axis=1)
    expect = (1 - np.exp(-sigma * g * dt * 1e20)).sum()
    assert cols == pytest.approx(expect, rel=5 * np.sqrt(expect) / expect)
    # oracle
    P = np.zeros((n, 12))
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = 1.0
    P[:, 10] = 1
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    z = np.zeros(nn)
    ocols = O.mcc(m, P, mass, mass, den, z, z, z, T, sigma, dt, 1, 3)
    assert cols == pytest.approx(ocols, rel=6 * np.sqrt(expect) / expect)
    # collided ions take the neutral temperature: their mean velocity drops to ~0
    changed = np.any(np.abs(v_after - vel) > 1e-3, axis=1)
    assert abs(changed.sum() - cols) <= 2
    assert abs(v_after[changed, 0].mean()) < 100.0


def test_mcc_ionization_matches_oracle(gpulib):
    """ModelIonization (MCC.java:304-356) on the GPU against the oracle: 50 eV electrons in a
    1e20 m^-3 argon background.  Collision count and ions per collision agree within their
    binomial spread; every collided electron has made one new electron of its own speed;
    energies and the ion Maxwellian match; delta_n, count and weight sums are exact; S
    agrees with the oracle's within its sampling spread."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, MCC
    spec = box_mesh()
    n, eV, e_ion = 200000, 50.0, 15.76
    me, mi, QE = 9.10938e-31, 40 * AMU, 1.60217646e-19
    spwt_e, spwt_i = 2.5e6, 1e6
    rng = np.random.default_rng(12)
    lc = rng.uniform(0.5, 19.5, (n, 2))
    lc = np.floor(lc) + (lc - np.floor(lc)).astype(np.float32).astype(np.float64)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    vel = (d * np.sqrt(2 * eV * QE / me)).astype(np.float32).astype(np.float64)
    nn = spec.nn
    den, T = np.full(nn, 1e20), np.full(nn, 300.0)
    sigma, dt = 1e-20, 5e-8
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(nn), np.zeros(nn))
        ke = KineticMaterial(dom, me, -QE, spwt_e, capacity=2 * n)
        ki = KineticMaterial(dom, mi, QE, spwt_i, capacity=2 * n)
        ke.add_particles_lc(lc, vel)
        mcc = MCC(dom, ke, target_mass=mi, den=den, temp=T, model=abi.MCC_IONIZATION,
                  sigma_model=abi.SIGMA_CONST, c=[sigma, 0, 0, 0])
        cols, n_e, n_i = mcc.perform(dt, product=ki, ionization_energy=e_ion)
        sums = mcc.sums()
        glc, gvel = ke.download()
        _, ivel = ki.download()
        assert ke.get_np() == n + n_e and ki.get_np() == n_i
    finally:
        dom.close()
    # oracle on the same electrons
    P = np.zeros((n, 12))
    P[:, 0:2] = spec.x0 + lc * spec.dh
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = spwt_e
    P[:, 10] = 1
    z = np.zeros(nn)
    o = O.mcc_ex(_om(spec), P, me, mi, den, z, z, z, T, sigma, dt, 2, 4, src_spwt=spwt_e, e_ion=e_ion,
                 prod_mass=mi, prod_spwt=spwt_i, max_new=4 * n)
    g = np.linalg.norm(vel, axis=1)
    expect = (1 - np.exp(-sigma * g * dt * 1e20)).sum()
    tol = 6 * np.sqrt(expect)
    assert abs(cols - expect) < tol and abs(o["cols"] - expect) < tol
    assert n_e == cols and o["n_new_e"] == o["cols"]
    assert abs(n_i / cols - 2.5) < 6 * 0.5 / np.sqrt(cols)
    # slots 0..n-1 are the original electrons, n.. the new ones
    v_src = gvel[:n]
    changed = np.any(np.abs(v_src - vel) > 1e-3 * np.abs(vel).max(), axis=1)
    assert abs(changed.sum() - cols) <= 2
    s_after = np.sort(np.linalg.norm(v_src[changed], axis=1))
    s_new = np.sort(np.linalg.norm(gvel[n:], axis=1))
    assert s_after.shape == s_new.shape
    assert np.allclose(s_new, s_after, rtol=2e-6)
    e_after = 0.5 * me * s_after ** 2 / QE
    assert e_after.max() <= eV - e_ion + 1e-3
    e_o = 0.5 * me * np.linalg.norm(o["new_e"][:, 3:6], axis=1) ** 2 / QE
    assert abs(e_after.mean() - e_o.mean()) < 6 * (eV - e_ion) / np.sqrt(12 * cols)
    sig_i = 1.2 * np.sqrt(2 * KB * 300 / mi) / np.sqrt(2)
    assert abs(ivel.std() / sig_i - 1) < 0.02 and abs(o["new_i"][:, 3:6].std() / sig_i - 1) < 0.02
    assert sums["delta_n"].sum() == pytest.approx(spwt_i * n_i, rel=1e-12)
    assert sums["count_sum"].sum() == cols
    assert sums["real_sum"].sum() == pytest.approx(spwt_e * cols, rel=1e-12)
    assert sums["S"].sum() == pytest.approx(o["S"].sum(), rel=6 / np.sqrt(cols))


def test_mcc_ionization_capacity_error(gpulib):
    """Products past the ion species' capacity: SF_ERR_OOM, and the count stops at it."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, MCC
    spec = box_mesh()
    n, QE, me = 20000, 1.60217646e-19, 9.10938e-31
    rng = np.random.default_rng(3)
    lc = rng.uniform(0.5, 19.5, (n, 2))
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    vel = d * np.sqrt(2 * 50 * QE / me)
    nn = spec.nn
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(nn), np.zeros(nn))
        ke = KineticMaterial(dom, me, -QE, 1e6, capacity=2 * n)
        ki = KineticMaterial(dom, 40 * AMU, QE, 1e6, capacity=100)
        ke.add_particles_lc(lc, vel)
        mcc = MCC(dom, ke, target_mass=40 * AMU, den=np.full(nn, 1e26), temp=np.full(nn, 300.0),
                  model=abi.MCC_IONIZATION, sigma_model=abi.SIGMA_CONST, c=[1e-20, 0, 0, 0])
        with pytest.raises(abi.SfError) as e:
            mcc.perform(5e-8, product=ki, ionization_energy=15.76)
        assert e.value.code == abi.SF_ERR_OOM
        assert ki.get_np() == 100
    finally:
        dom.close()
