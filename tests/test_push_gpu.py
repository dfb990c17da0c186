"""GPU parity of the push + scatter (KineticMaterial.updateFields) against the oracle.

Identical particle state is loaded into both (logical coordinates that FP32 holds
exactly, FP32-representable velocities); one step is taken; survivors, positions,
velocities, node densities, ParticleMover totals and surface deposits are compared.
Tolerances: positions 1e-5 cells absolute, velocities 1e-6 relative, densities
1e-6 of the field maximum (the push runs in FP32, the oracle in FP64).
"""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _omesh(spec):
    return O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)


def make_state(spec, ion, n, seed, fast_fraction=0.05):
    """Random particles outside the electrode; a few fast ones cross several cells."""
    pos, vel = W.uniform_maxwellian(spec, ion, n, seed)
    rng = np.random.default_rng(seed + 1)
    k = int(n * fast_fraction)
    vel[:k] *= rng.uniform(2, 6, (k, 1))
    lc = np.empty((n, 2))
    lc[:, 0] = (pos[:, 0] - spec.x0[0]) / spec.dh[0]
    lc[:, 1] = (pos[:, 1] - spec.x0[1]) / spec.dh[1]
    # make the state exactly representable as (int cell, FP32 fraction), FP32 velocity
    i = np.minimum(np.floor(lc[:, 0]), spec.ni - 2)
    j = np.minimum(np.floor(lc[:, 1]), spec.nj - 2)
    lc[:, 0] = i + (lc[:, 0] - i).astype(np.float32).astype(np.float64)
    lc[:, 1] = j + (lc[:, 1] - j).astype(np.float32).astype(np.float64)
    vel = vel.astype(np.float32).astype(np.float64)
    return lc, vel


def oracle_parts(spec, lc, vel, spwt):
    n = lc.shape[0]
    P = np.zeros((n, 12))
    P[:, 0] = spec.x0[0] + lc[:, 0] * spec.dh[0]
    P[:, 1] = spec.x0[1] + lc[:, 1] * spec.dh[1]
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = spwt
    P[:, 10] = 1
    return P


def run_case(spec, ion, n, seed, dt, efi, efj):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    lc, vel = make_state(spec, ion, n, seed)
    dom = GpuDomain(spec)
    dom.set_efield(efi, efj)
    km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=n + 16)
    km.set_sort_interval(0)      # keep storage order for a particle-by-particle comparison
    km.add_particles_lc(lc, vel)
    st = km.update_fields(dt, stats=True)
    glc, gvel = km.download()
    gden = km.get_den()
    gflux, gdep = km.surface_flux()

    m = _omesh(spec)
    # E as the GPU holds it (FP32) so that both start from the same field
    e32i = efi.astype(np.float32).astype(np.float64)
    e32j = efj.astype(np.float32).astype(np.float64)
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_ABSORB)
    P = oracle_parts(spec, lc, vel, ion.spwt)
    alive, ost, oflux, odep = O.push(m, e32i, e32j, ion.charge, ion.mass, dt, segs,
                                     spec.node_seg_ptr, spec.node_seg_idx, P)
    vol = O.node_volumes(m)
    oden = O.update_fields(m, vol, P)
    dom.close()
    return dict(glc=glc, gvel=gvel, gden=gden, st=st, gflux=gflux, gdep=gdep, P=P, alive=alive,
                ost=ost, oflux=oflux, odep=odep, oden=oden)


@pytest.mark.parametrize("seed", [0, 1])
def test_push_deposit_matches_oracle_c0(gpulib, seed):
    spec = W.es_pic_mesh(81, 41, 1e-3)
    ion = W.IonSpecies()
    _, efi, efj = W.electrode_efield(spec)
    r = run_case(spec, ion, 20000, seed, 5e-7, efi, efj)
    P = r["P"]
    keep = P[:, 10] == 1
    assert r["alive"] == keep.sum()
    assert r["glc"].shape[0] == keep.sum()
    assert r["st"]["np"] == keep.sum()
    # survivors in storage order
    olc = P[keep, 6:8]
    ovel = P[keep, 3:6]
    assert np.max(np.abs(r["glc"] - olc)) < 1e-5
    vscale = np.linalg.norm(ovel, axis=1, keepdims=True)
    assert np.max(np.abs(r["gvel"] - ovel) / vscale) < 1e-6
    dmax = np.abs(r["oden"]).max()
    assert np.max(np.abs(r["gden"] - r["oden"])) <= 1e-6 * dmax
    # ParticleMover totals (per weight) and the surface mass deposit
    assert r["st"]["n_sum"] == pytest.approx(r["ost"][0] * 1.0, rel=1e-12)
    for d in range(3):
        assert r["st"]["p_sum"][d] == pytest.approx(r["ost"][1 + d], rel=1e-5, abs=1e-5 * r["ost"][4])
    assert r["st"]["e_sum"] == pytest.approx(r["ost"][4], rel=1e-5)
    # absorbed weight per segment is exact; its split over the segment ends follows the
    # hit point, which moves with the FP32 velocity update (1e-8 relative)
    seg_g = r["gdep"].reshape(-1, 2).sum(axis=1)
    seg_o = r["odep"].reshape(-1, 2).sum(axis=1)
    assert np.allclose(seg_g, seg_o, rtol=1e-12)
    assert np.allclose(r["gdep"], r["odep"], rtol=1e-6)
    assert r["st"]["n_slow"] > 0 and r["st"]["n_removed"] > 0


def test_push_symmetry_and_open_faces(gpulib):
    """Bottom symmetry (mirror), right open, left/top Dirichlet walls (deleted)."""
    spec = W.es_pic_mesh(61, 31, 1e-3, electrode_halfwidth=3e-3)
    spec.face_type[abi.FACE_BOTTOM, :] = abi.DB_SYMMETRY
    spec.face_type[abi.FACE_RIGHT, :] = abi.DB_OPEN
    ion = W.IonSpecies(v_drift=-3000.0)
    _, efi, efj = W.electrode_efield(spec)
    efj = efj - 2e3   # push ions into the bottom face (0.1 cell per step extra)
    r = run_case(spec, ion, 20000, 5, 5e-7, efi, efj)
    P = r["P"]
    keep = P[:, 10] == 1
    assert r["glc"].shape[0] == keep.sum()
    assert np.max(np.abs(r["glc"] - P[keep, 6:8])) < 1e-5
    vs = np.linalg.norm(P[keep, 3:6], axis=1, keepdims=True)
    assert np.max(np.abs(r["gvel"] - P[keep, 3:6]) / vs) < 1e-6
    assert np.max(np.abs(r["gden"] - r["oden"])) <= 1e-6 * np.abs(r["oden"]).max()


def test_deposit_bit_reproducible(gpulib):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(257, 129, 2.5e-4, electrode_halfwidth=4.5e-3)
    ion = W.IonSpecies()
    _, efi, efj = W.electrode_efield(spec)
    pos, vel = W.uniform_maxwellian(spec, ion, 400000, 3)
    outs = []
    for rep in range(2):
        dom = GpuDomain(spec)
        dom.set_efield(efi, efj)
        km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=500000)
        km.add_particles(pos, vel, rewind=True, dt=1.25e-7)
        for _ in range(3):
            km.update_fields(1.25e-7)
        outs.append((km.get_count(), km.get_den()))
        dom.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_deposit_conserves_weight(gpulib):
    """Sum over nodes of the deposited weight equals the particles' weight (fixed point
    rounding <= 2 units of 2^-31 per particle)."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(513, 257, 2e-4, electrode_halfwidth=4.5e-3, walls=abi.DB_OPEN)
    spec.seg_xy = np.zeros((0, 4))
    spec.seg_btype = np.zeros(0, np.int32)
    spec.node_type[:] = abi.NODE_OPEN
    ion = W.IonSpecies(v_drift=0.0)
    efi = np.zeros(spec.nn)
    efj = np.zeros(spec.nn)
    rng = np.random.default_rng(9)
    n = 2_000_000
    lc = np.column_stack([rng.uniform(2, spec.ni - 3, n), rng.uniform(2, spec.nj - 3, n)])
    vel = rng.normal(0, 10.0, (n, 3))
    dom = GpuDomain(spec)
    dom.set_efield(efi, efj)
    km = KineticMaterial(dom, ion.mass, ion.charge, 1.0, capacity=n)
    km.add_particles_lc(lc, vel)
    st = km.update_fields(1e-9)
    assert st["np"] == n and st["n_removed"] == 0
    total = km.get_count().sum()
    assert abs(total - n) <= 2 * n * 2.0 ** -31 * 4 + 1e-6
    dom.close()


def _tile_key(lc, ni, nj):
    i = np.minimum(np.floor(lc[:, 0]).astype(np.int64), ni - 2)
    j = np.minimum(np.floor(lc[:, 1]).astype(np.int64), nj - 2)
    ntx = (ni - 1 + 15) // 16
    return (((j >> 4) * ntx + (i >> 4)) << 8) | ((j & 15) << 4) | (i & 15)


def test_cell_sort_orders_and_keeps_particles(gpulib):
    """The counting sort (DSMC.perform(mesh) binning, DSMC.java:194-231) keeps every
    particle, drops removed ones and leaves cell keys in non-decreasing order."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(301, 151, 1e-3, electrode_halfwidth=1e-2)
    ion = W.IonSpecies()
    _, efi, efj = W.electrode_efield(spec)
    pos, vel = W.uniform_maxwellian(spec, ion, 300000, 11)
    dom = GpuDomain(spec)
    dom.set_efield(efi, efj)
    km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=400000)
    km.set_sort_interval(0)
    km.add_particles(pos, vel, rewind=False)
    lc0, v0 = km.download()
    km.update_fields(5e-7)          # removes some particles (electrode, walls)
    lc1, v1 = km.download()
    km.sort()
    lc2, v2 = km.download()
    km.sort()                       # sorted input: whole warps share a cell key
    lc3, v3 = km.download()
    dom.close()
    assert lc2.shape[0] == lc1.shape[0] < lc0.shape[0]
    a = np.lexsort(np.column_stack([lc1, v1]).T)
    for lc, v in ((lc2, v2), (lc3, v3)):
        k = _tile_key(lc, spec.ni, spec.nj)
        assert np.all(np.diff(k) >= 0)
        b = np.lexsort(np.column_stack([lc, v]).T)
        assert np.array_equal(np.column_stack([lc1, v1])[a], np.column_stack([lc, v])[b])


@pytest.mark.parametrize("cells", [2, 4, 16])
def test_sort_block_changes_order_only(gpulib, cells):
    """The automatic sort's key block (sf_species_set_sort_block) only reorders: pushes
    with sorts by 1-cell and by coarser key blocks (look-ahead keys, a sort every other
    push) give bit-identical node counts and the same surviving particles."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(257, 129, 2.5e-4, electrode_halfwidth=4.5e-3)
    ion = W.IonSpecies()
    _, efi, efj = W.electrode_efield(spec)
    pos, vel = W.uniform_maxwellian(spec, ion, 300000, 5)
    outs = []
    for b in (1, cells):
        dom = GpuDomain(spec)
        dom.set_efield(efi, efj)
        km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=400000)
        km.set_sort_interval(2)
        km.set_sort_block(b)
        km.add_particles(pos, vel, rewind=True, dt=1.25e-7)
        counts = []
        for _ in range(5):
            km.update_fields(1.25e-7)
            counts.append(km.get_count())
        lc, v = km.download()
        outs.append((counts, lc, v))
        dom.close()
    for c0, c1 in zip(outs[0][0], outs[1][0]):
        assert np.array_equal(c0, c1)
    (_, lc0, v0), (_, lc1, v1) = outs
    assert lc0.shape == lc1.shape
    a = np.lexsort(np.column_stack([lc0, v0]).T)
    b_ = np.lexsort(np.column_stack([lc1, v1]).T)
    assert np.array_equal(np.column_stack([lc0, v0])[a], np.column_stack([lc1, v1])[b_])


def test_sort_block_rejects_bad_sizes(gpulib):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(81, 41, 1e-3)
    ion = W.IonSpecies()
    dom = GpuDomain(spec)
    km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=100)
    for bad in (0, 3, 32, -1):
        with pytest.raises(abi.SfError):
            km.set_sort_block(bad)
    dom.close()
