"""Device particle sources against the oracle, and a restart round trip.

VolumePreloadSource (sf_source_preload) and UniformSource (sf_source_uniform) draw from
Philox streams, the oracle from java.util.Random, so counts that involve random positions
are compared within their sampling spread and the deterministic parts exactly.  The
restart test downloads a species and loads it into a fresh context (sf_particles_download,
sf_particles_append_lc): the two must then push identically, bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

AMU = 1.66053886e-27
KB = 1.3806503e-23


def test_preload_matches_oracle(gpulib):
    """Count per cell ceil(den V / spwt) - 1 minus the points inside the electrode; no
    particle inside; Maxwellian at temp with the sampler's 1.2 factor; uniform in space."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(81, 41, 1e-3)
    mass, spwt, den, T, dt = 16 * AMU, 2000.0, 1e12, 1000.0, 5e-7
    nn = spec.nn
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(nn), np.zeros(nn))
        km = KineticMaterial(dom, mass, 1.602e-19, spwt, capacity=2_000_000)
        added = km.preload(den, T, dt)
        lc, vel = km.download()
    finally:
        dom.close()
    o = O.preload(7, spec, den, T, mass, spwt, dt, cap=2_000_000)
    per_cell = int(np.ceil(den * 1e-6 / spwt)) - 1
    total = per_cell * 80 * 40
    inside = total * (9e-3 * 9e-3) / (80e-3 * 40e-3)
    tol = 6 * np.sqrt(inside)
    assert abs(added - (total - inside)) < tol and abs(o.shape[0] - (total - inside)) < tol
    assert lc.shape[0] == added
    pos = spec.x0 + lc * spec.dh
    sample = pos[:: max(1, added // 3000)]
    assert not any(O.point_internal(spec.seg_xy, spec.seg_btype, x, y) for x, y in sample)
    sig = 1.2 * np.sqrt(2 * KB * T / mass) / np.sqrt(2)
    assert abs(vel.std() / sig - 1) < 0.01 and abs(o[:, 3:6].std() / sig - 1) < 0.01
    assert abs(vel.mean()) < 5 * sig / np.sqrt(vel.size)
    # uniform in space: the x histogram over the gas columns is flat
    cols = np.histogram(pos[:, 0], bins=80, range=(0, 0.08))[0]
    gas = np.r_[cols[:34], cols[46:]]
    assert gas.std() / gas.mean() < 0.02


def test_uniform_source_matches_oracle(gpulib):
    """Counts of Source.regenerate over several calls (the remainder carried), the cold
    beam v = normal * v_drift, positions spread evenly along the segment."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(81, 41, 1e-3)
    mass, spwt, dt = 16 * AMU, 1e3, 5e-7
    mdot, v = 3.3e-13, 6000.0
    seg = np.array([0.0, 0.04, 0.0, 0.0])
    nn = spec.nn
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(nn), np.zeros(nn))
        km = KineticMaterial(dom, mass, 1.602e-19, spwt, capacity=4_000_000)
        counts = [km.sample_uniform_source(seg, mdot, v, dt) for _ in range(5)]
        lc, vel = km.download()
    finally:
        dom.close()
    rem, ocounts = 0.0, []
    for k in range(5):
        p, rem = O.uniform_source(k, seg, mdot, v, mass, spwt, dt, rem=rem)
        ocounts.append(p.shape[0])
    assert counts == ocounts
    assert np.all(vel[:, 0] == np.float32(v)) and np.all(vel[:, 1:] == 0)
    y = spec.x0[1] + lc[:, 1] * spec.dh[1]
    assert abs(y.mean() - 0.02) < 6 * 0.04 / np.sqrt(12 * y.size)
    x = spec.x0[0] + lc[:, 0] * spec.dh[0]
    assert np.allclose(x, v * 1e-6 * dt, rtol=1e-3)


def test_restart_round_trip(gpulib):
    """A species downloaded and loaded into a fresh context pushes exactly as the original."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    cfg = W.config0()
    spec, ion = cfg.mesh, cfg.ion
    _, efi, efj = W.electrode_efield(spec)
    pos, vel = W.uniform_maxwellian(spec, ion, 200_000, 5)
    doms = [GpuDomain(spec), GpuDomain(spec)]
    try:
        for d in doms:
            d.set_efield(efi, efj)
        a = KineticMaterial(doms[0], ion.mass, ion.charge, ion.spwt, capacity=400_000)
        a.add_particles(pos, vel, rewind=True, dt=cfg.dt)
        for _ in range(3):
            a.update_fields(cfg.dt, stats=False)
        lc, v = a.download()  # the restart file's content
        b = KineticMaterial(doms[1], ion.mass, ion.charge, ion.spwt, capacity=400_000)
        b.add_particles_lc(lc, v)
        la, va = a.download()
        lb, vb = b.download()
        assert np.array_equal(la, lb) and np.array_equal(va, vb)
        a.update_fields(cfg.dt, stats=False)
        b.update_fields(cfg.dt, stats=False)
        assert np.array_equal(a.get_den(), b.get_den())
        la, va = a.download()
        lb, vb = b.download()
        sa, sb = np.lexsort(np.hstack([la, va]).T), np.lexsort(np.hstack([lb, vb]).T)
        assert np.array_equal(la[sa], lb[sb]) and np.array_equal(va[sa], vb[sb])
    finally:
        for d in doms:
            d.close()
