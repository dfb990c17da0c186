"""Edge cases of the push, sort and collision paths: an empty species, a population that
leaves the mesh in one push, ragged particle counts around the push tile (1024 particles)
and the sort chunk, and a DSMC call on an empty species.  The reference handles all of them
as plain loops over its particle lists (KineticMaterial.java:117-197, DSMC.java:162-192)."""
import numpy as np
import pytest

from oracle import oracle as O
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


def test_empty_species_push_sort_dsmc(gpulib):
    from starfish_gb300.plugin import DSMC, GpuDomain, KineticMaterial
    spec = _open_box()
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, 40 * 1.6605e-27, 0.0, 1e10, capacity=1024)
        for _ in range(3):
            st = km.update_fields(1e-7, stats=True)
            assert st["np"] == 0 and st["n_removed"] == 0
        km.sort()
        assert km.get_np() == 0
        assert not km.get_count().any()
        assert not km.get_den().any()
        d = DSMC(dom, km, diam=4.17e-10, omega=0.81)
        assert d.perform(1e-6) == 0
        lc, vel = km.download()
        assert lc.shape[0] == 0
    finally:
        dom.close()


def test_population_that_leaves_in_one_push(gpulib):
    """Every particle crosses an open face in the first push: all are removed, the density
    is zero, the next sort keeps nothing and later pushes and appends work."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = _open_box()
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, 16 * 1.6605e-27, 1.602e-19, 1e5, capacity=5000)
        n = 3000
        rng = np.random.default_rng(2)
        lc = np.column_stack([rng.uniform(spec.ni - 1.5, spec.ni - 1.01, n), rng.uniform(1, spec.nj - 2, n)])
        vel = np.zeros((n, 3))
        vel[:, 0] = 5.0 * spec.dh[0] / 1e-7  # five cells per step along +x
        km.add_particles_lc(lc, vel)
        st = km.update_fields(1e-7, stats=True)
        assert st["n_removed"] == n and st["np"] == 0
        assert not km.get_count().any()
        km.sort()
        assert km.get_np() == 0
        km.add_particles_lc(lc[:10] - [spec.ni // 2, 0], np.zeros((10, 3)))
        st = km.update_fields(1e-7, stats=True)
        assert st["np"] == 10
    finally:
        dom.close()


@pytest.mark.parametrize("n", [1, 31, 1023, 1024, 1025, 2049, 4097])
def test_ragged_counts_match_oracle(gpulib, n):
    """Particle counts around the push tile and the sort chunk: the deposit and the moved
    particles against the oracle's push and scatter of the same state."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = _open_box(65, 33)
    rng = np.random.default_rng(n)
    efi = rng.normal(0, 50, spec.nn)
    efj = rng.normal(0, 50, spec.nn)
    lc = np.column_stack([rng.uniform(3, spec.ni - 4, n), rng.uniform(3, spec.nj - 4, n)])
    i = np.floor(lc[:, 0])
    j = np.floor(lc[:, 1])
    lc[:, 0] = i + (lc[:, 0] - i).astype(np.float32).astype(np.float64)
    lc[:, 1] = j + (lc[:, 1] - j).astype(np.float32).astype(np.float64)
    vel = rng.normal(0, 300.0, (n, 3)).astype(np.float32).astype(np.float64)
    q, mass, spwt, dt = 1.602e-19, 16 * 1.6605e-27, 1e5, 1e-7
    dom = GpuDomain(spec)
    try:
        dom.set_efield(efi, efj)
        km = KineticMaterial(dom, mass, q, spwt, capacity=n + 64)
        km.set_sort_interval(0)
        km.add_particles_lc(lc, vel)
        st = km.update_fields(dt, stats=True)
        glc, gvel = km.download()
        gden = km.get_den()
    finally:
        dom.close()
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    P = np.zeros((n, 12))
    P[:, 0] = spec.x0[0] + lc[:, 0] * spec.dh[0]
    P[:, 1] = spec.x0[1] + lc[:, 1] * spec.dh[1]
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = spwt
    P[:, 10] = 1
    segs = O.seg_table(np.zeros((0, 4)), np.zeros(0, np.int32), O.SURF_ABSORB)
    e32i = efi.astype(np.float32).astype(np.float64)
    e32j = efj.astype(np.float32).astype(np.float64)
    O.push(m, e32i, e32j, q, mass, dt, segs, spec.node_seg_ptr, spec.node_seg_idx, P)
    keep = P[:, 10] == 1
    assert st["np"] == keep.sum() == n
    oden = O.update_fields(m, O.node_volumes(m), P)
    assert np.max(np.abs(gden - oden)) <= 1e-6 * np.abs(oden).max()
    assert np.max(np.abs(glc - P[:, 6:8])) < 1e-5
    vs = np.abs(P[:, 3:6]).max()
    assert np.max(np.abs(gvel - P[:, 3:6])) < 1e-6 * vs
