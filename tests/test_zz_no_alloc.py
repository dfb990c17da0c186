"""sf_push_deposit_noalloc (push scratch in a static device array) against sf_push_deposit.

Two contexts hold identical particles and the same field; one steps with the ordinary
entry point, the other with the no-allocation one, twice in a row, so that the second
call runs on scratch that still holds the first call's contents.  After each call the
densities, moments, ParticleMover totals, counters and particle states must agree to
the push parity tolerances (densities 1e-6 of the field maximum, positions 1e-5 cells,
velocities 1e-6 relative, totals 1e-5); the deposit is integer fixed point, so the
densities agree exactly in practice.  The driver's free-memory figure must not move
across any no-allocation call, including the first one, which also cell-sorts the freshly
appended particles.  The file sorts last so that it also runs after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NOALLOC_MAX_PARTICLES = 1 << 21


def _state(spec, ion, n, seed):
    pos, vel = W.uniform_maxwellian(spec, ion, n, seed)
    rng = np.random.default_rng(seed + 7)
    k = n // 10
    vel[:k] *= rng.uniform(2, 6, (k, 1))  # fast ones reach the electrode and the walls
    return pos, vel


def _species(dom, ion, pos, vel, dt):
    from starfish_gb300.plugin import KineticMaterial
    km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=pos.shape[0] + 16)
    km.add_particles(pos, vel, rewind=True, dt=dt)
    return km


def _step(dom, km, dt, noalloc):
    st = abi.PushStats()
    fn = dom.lib.sf_push_deposit_noalloc if noalloc else dom.lib.sf_push_deposit
    rc = fn(dom.ctx, km.sid, C.c_double(dt), abi.PUSH_STATS | abi.PUSH_MOMENTS, C.byref(st))
    dom.check(rc)
    return st.as_dict()


def _compare(dom_a, km_a, st_a, dom_b, km_b, st_b):
    for key in ("np", "n_removed", "n_slow", "n_bounce_limited"):
        assert st_a[key] == st_b[key], key
    # totals: the push tests' tolerances (the slow path sums with floating-point atomics,
    # so the last bits follow the order, as between two calls of the same entry point)
    assert st_b["n_sum"] == pytest.approx(st_a["n_sum"], rel=1e-12)
    assert st_b["e_sum"] == pytest.approx(st_a["e_sum"], rel=1e-5)
    assert st_b["boundary_charge"] == pytest.approx(st_a["boundary_charge"], rel=1e-6)
    for d in range(3):
        assert st_b["p_sum"][d] == pytest.approx(st_a["p_sum"][d], rel=1e-5, abs=1e-5 * max(map(abs, st_a["p_sum"])))
    den_a, den_b = km_a.get_den(), km_b.get_den()
    assert np.max(np.abs(den_a - den_b)) <= 1e-6 * np.max(np.abs(den_a))
    for ua, ub in zip(km_a.get_uvw(), km_b.get_uvw()):
        assert np.max(np.abs(ua - ub)) <= 1e-6 * max(np.max(np.abs(ua)), 1e-30)
    # the cell sort orders particles within a cell by arrival, so compare the particle
    # sets: rows of (lc, v) in lexicographic order
    pa, pb = np.hstack(km_a.download()), np.hstack(km_b.download())
    assert pa.shape == pb.shape
    pa = pa[np.lexsort(pa.T[::-1])]
    pb = pb[np.lexsort(pb.T[::-1])]
    assert np.max(np.abs(pa[:, :2] - pb[:, :2]), initial=0.0) <= 1e-5
    assert np.max(np.abs(pa[:, 2:] - pb[:, 2:]), initial=0.0) <= 1e-6 * np.max(np.abs(pa[:, 2:]))


def _device_free_bytes():
    """Free memory of the current device as the driver reports it (cudaMemGetInfo): any
    cudaMalloc, by the library or anyone else in the process, lowers it."""
    torch = pytest.importorskip("torch")
    free, _ = torch.cuda.mem_get_info()
    return free


def test_noalloc_push_matches_push_two_calls(gpulib):
    """Also checks that no call of the no-allocation entry point changes the device's free
    memory: the first one, which runs the automatic cell sort of the freshly appended
    species, and the second.  The ordinary entry point runs first on its own context, so
    the kernels both use are already loaded when the no-allocation calls are measured."""
    from starfish_gb300.plugin import GpuDomain
    cfg = W.config0()
    spec, ion = cfg.mesh, cfg.ion
    _, efi, efj = W.electrode_efield(spec)
    pos, vel = _state(spec, ion, 200_000, seed=11)
    dom_a, dom_b = GpuDomain(spec), GpuDomain(spec)
    try:
        for d in (dom_a, dom_b):
            d.set_efield(efi, efj)
        km_a = _species(dom_a, ion, pos, vel, cfg.dt)
        km_b = _species(dom_b, ion, pos, vel, cfg.dt)
        _device_free_bytes()  # the query's own set-up happens before the first reading
        for call in range(2):
            st_a = _step(dom_a, km_a, cfg.dt, noalloc=False)
            free0 = _device_free_bytes()
            st_b = _step(dom_b, km_b, cfg.dt, noalloc=True)
            free1 = _device_free_bytes()
            assert free1 == free0, f"call {call}: free device memory changed by {free0 - free1} bytes"
            assert st_a["n_slow"] > 0 and st_a["n_removed"] > 0, "the case must exercise the slow path"
            _compare(dom_a, km_a, st_a, dom_b, km_b, st_b)
    finally:
        dom_a.close()
        dom_b.close()


def test_noalloc_push_rejects_oversized_species(gpulib):
    from starfish_gb300.plugin import GpuDomain
    cfg = W.config0()
    spec, ion = cfg.mesh, cfg.ion
    dom = GpuDomain(spec)
    try:
        dom.set_efield(*W.electrode_efield(spec)[1:])
        n = NOALLOC_MAX_PARTICLES + 1
        pos, vel = W.uniform_maxwellian(spec, ion, n, seed=3)
        km = _species(dom, ion, pos, vel, cfg.dt)
        st = abi.PushStats()
        rc = dom.lib.sf_push_deposit_noalloc(dom.ctx, km.sid, C.c_double(cfg.dt), 0, C.byref(st))
        assert rc == abi.SF_ERR_ARG
        msg = dom.lib.sf_last_error(dom.ctx).decode()
        assert "2097152" in msg and "sf_push_deposit" in msg
        assert km.get_np() == n  # rejected before any work
    finally:
        dom.close()
