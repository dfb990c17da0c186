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
