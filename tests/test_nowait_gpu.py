"""Pushes that do not wait (SF_PUSH_NOWAIT) against pushes that do: the same particles,
densities and counts, with automatic sorts and appends between them; the particle-steps
counter against the per-step counts; and the no-allocation entry point, which waits
for every call, refusing the flag."""
import ctypes as C

import numpy as np
import pytest

from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _open_box(ni=129, nj=65, dh=1e-3):
    spec = W.es_pic_mesh(ni, nj, dh, walls=abi.DB_OPEN)
    spec.seg_xy = np.zeros((0, 4))
    spec.seg_btype = np.zeros(0, np.int32)
    spec.node_type[:] = abi.NODE_OPEN
    spec.bc_value[:] = 0.0
    return spec


def _state(n, spec, seed):
    rng = np.random.default_rng(seed)
    lc = np.column_stack([rng.uniform(1, spec.ni - 2, n), rng.uniform(1, spec.nj - 2, n)])
    vel = rng.normal(0, 2000.0, (n, 3))
    vel[:, 0] += 3000.0  # a drift towards the open x = max face: particles leave every step
    return lc, vel


def _sorted(lc, vel):
    a = np.column_stack([lc, vel])
    return a[np.lexsort(a.T[::-1])]


def test_nowait_matches_waiting_push(gpulib):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = _open_box()
    rng = np.random.default_rng(5)
    efi = rng.normal(0, 200, spec.nn)
    efj = rng.normal(0, 200, spec.nn)
    lc0, vel0 = _state(200_000, spec, 11)
    lc1, vel1 = _state(5_000, spec, 12)
    dt = 1e-7
    out = []
    for wait in (True, False):
        dom = GpuDomain(spec)
        try:
            dom.set_efield(efi, efj)
            km = KineticMaterial(dom, 16 * 1.6605e-27, 1.602e-19, 1e5, capacity=300_000)
            km.set_sort_interval(4)
            km.add_particles_lc(lc0, vel0)
            np_steps, removed = [], 0
            ps0 = km.particle_steps()
            for k in range(11):
                if wait:
                    np_steps.append(km.get_np())
                st = km.update_fields(dt, stats=False, wait=wait)
                if wait:
                    removed += st["n_removed"]
                else:
                    assert st["np"] == -1 and st["n_removed"] == -1
                if k == 6:
                    km.add_particles_lc(lc1, vel1)  # settles the counts of the pushes before
            psteps = km.particle_steps() - ps0
            out.append(dict(np=km.get_np(), den=km.get_den(), count=km.get_count(), psteps=psteps,
                            parts=_sorted(*km.download()), np_steps=np_steps, removed=removed))
        finally:
            dom.close()
    a, b = out
    assert a["removed"] > 1000  # the open face removes particles at every step
    assert a["np"] == b["np"] == 200_000 + 5_000 - a["removed"]
    assert a["psteps"] == b["psteps"] == sum(a["np_steps"])
    assert np.array_equal(a["den"], b["den"])
    assert np.array_equal(a["count"], b["count"])
    assert np.array_equal(a["parts"], b["parts"])


def test_nowait_with_stats_waits(gpulib):
    """SF_PUSH_STATS needs the push's results, so the flag is ignored there."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = _open_box()
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, 16 * 1.6605e-27, 1.602e-19, 1e5, capacity=10_000)
        lc, vel = _state(4096, spec, 3)
        km.add_particles_lc(lc, vel)
        km.update_fields(1e-7, stats=False, wait=False)
        st = km.update_fields(1e-7, stats=True, wait=False)
        assert st["np"] == km.get_np() and st["np"] > 0
    finally:
        dom.close()


def test_noalloc_refuses_nowait(gpulib):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = _open_box()
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, 16 * 1.6605e-27, 1.602e-19, 1e5, capacity=10_000)
        lc, vel = _state(1000, spec, 4)
        km.add_particles_lc(lc, vel)
        st = abi.PushStats()
        rc = dom.lib.sf_push_deposit_noalloc(dom.ctx, km.sid, 1e-7, abi.PUSH_NOWAIT, C.byref(st))
        assert rc == abi.SF_ERR_ARG
        assert km.get_np() == 1000
    finally:
        dom.close()


def test_dsmc_without_count_readback(gpulib):
    """sf_dsmc with n_coll NULL queues the collisions: the per-cell sums hold them, and a
    later call that reads its count sees the same cell state."""
    from starfish_gb300.plugin import DSMC, GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(33, 33, 1e-3, walls=abi.DB_SYMMETRY, electrode_halfwidth=1e-12)
    spec.seg_xy = np.zeros((0, 4))
    spec.seg_btype = np.zeros(0, np.int32)
    spec.node_type[:] = abi.NODE_OPEN
    spec.bc_value[:] = 0.0
    rng = np.random.default_rng(4)
    n = 64 * 32 * 32
    lc = rng.uniform(0.01, 31.99, (n, 2))
    vel = rng.normal(0, 300.0, (n, 3))
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, 40 * 1.6605e-27, 0.0, 1e13, capacity=n + 64)
        km.add_particles_lc(lc, vel)
        ds = DSMC(dom, km, model=abi.SIGMA_BIRD463, diam=4.17e-10, T_ref=273.0, omega=0.81)
        got = [ds.perform(1e-6, wait=False) for _ in range(3)]
        assert got == [None, None, None]
        c3 = ds.counts()[0].sum()
        assert c3 > 0
        nc = ds.perform(1e-6)
        assert nc > 0 and ds.counts()[0].sum() == c3 + nc
        assert km.get_np() == n
    finally:
        dom.close()


def test_source_without_count_readback(gpulib):
    """sf_source_maxwellian with n_added NULL: draw k takes slot n + k, a draw outside the
    mesh leaves its slot removed.  The particles equal those of the counted call as a set;
    the counts agree once read."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = _open_box(65, 33)
    # a segment reaching past the top of the mesh: part of the draws land outside
    seg = np.array([spec.x0[0] + 20e-3, spec.x0[1] + 40e-3, spec.x0[0] + 20e-3, spec.x0[1] + 10e-3])
    out = []
    for wait in (True, False):
        dom = GpuDomain(spec)
        try:
            dom.set_seed(7)
            dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
            km = KineticMaterial(dom, 16 * 1.6605e-27, 1.602e-19, 1e5, capacity=200_000)
            for _ in range(3):
                r = km.sample_maxwellian_source(seg, 1e12, 5000.0, 1000.0, 1e-7, wait=wait)
                assert (r is None) != wait
            out.append((km.get_np(), _sorted(*km.download())))
        finally:
            dom.close()
    (n0, p0), (n1, p1) = out
    assert 0 < n0 == n1
    assert np.array_equal(p0, p1)
