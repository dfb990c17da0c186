"""Per-particle weights (Particle.mpw, KineticMaterial.java:1207-1282): a species switched to
weights (sf_species_set_weighted) pushes, scatters, sums and hits surfaces with each
particle's own mpw, against the oracle, which carries mpw per particle as the reference
does; the weights follow their particles through the sort and the restart path; sources
on a weighted species emit at the species weight; DSMC and MCC take each particle's
weight.  The batched instances with weighted species are checked in test_batch_gpu.py."""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

from test_push_gpu import make_state, oracle_parts  # noqa: E402


def _omesh(spec):
    return O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)


@pytest.mark.parametrize("seed", [1, 2])
def test_weighted_push_matches_oracle_c0(gpulib, seed):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(81, 41, 1e-3)
    ion = W.IonSpecies()
    _, efi, efj = W.electrode_efield(spec)
    n, dt = 20000, 5e-7
    lc, vel = make_state(spec, ion, n, seed)
    rng = np.random.default_rng(seed + 50)
    # weights that FP32 holds exactly as fractions of spwt
    frac = np.round(rng.uniform(0.25, 1.0, n) * 256) / 256
    mpw = frac * ion.spwt
    dom = GpuDomain(spec)
    try:
        dom.set_efield(efi, efj)
        km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=n + 16)
        km.set_weighted(True)
        km.set_sort_interval(0)
        km.add_particles_lc(lc, vel, mpw=mpw)
        st = km.update_fields(dt, stats=True)
        glc, gvel = km.download()
        gw = km.download_weights()
        gden = km.get_den()
        gflux, gdep = km.surface_flux()
    finally:
        dom.close()
    m = _omesh(spec)
    e32i = efi.astype(np.float32).astype(np.float64)
    e32j = efj.astype(np.float32).astype(np.float64)
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_ABSORB)
    P = oracle_parts(spec, lc, vel, ion.spwt)
    P[:, 9] = mpw
    alive, ost, oflux, odep = O.push(m, e32i, e32j, ion.charge, ion.mass, dt, segs,
                                     spec.node_seg_ptr, spec.node_seg_idx, P)
    oden = O.update_fields(m, O.node_volumes(m), P)
    keep = P[:, 10] == 1
    assert st["np"] == keep.sum() == glc.shape[0]
    assert np.max(np.abs(glc - P[keep, 6:8])) < 1e-5
    assert np.array_equal(gw, mpw[keep])
    # the weighted density: each corner share quantised as 2^-22 of the species weight
    assert np.max(np.abs(gden - oden)) <= 1e-6 * np.abs(oden).max()
    assert st["n_sum"] == pytest.approx(ost[0], rel=1e-6)
    assert st["e_sum"] == pytest.approx(ost[4], rel=1e-5)
    seg_g = gdep.reshape(-1, 2).sum(axis=1)
    seg_o = odep.reshape(-1, 2).sum(axis=1)
    assert np.allclose(seg_g, seg_o, rtol=1e-12)
    assert np.allclose(gdep, odep, rtol=1e-6)
    assert st["n_removed"] > 0


def test_weights_follow_particles_through_sort_and_restart(gpulib):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(257, 129, 2.5e-4, electrode_halfwidth=4.5e-3)
    ion = W.IonSpecies()
    _, efi, efj = W.electrode_efield(spec)
    pos, vel = W.uniform_maxwellian(spec, ion, 200000, 7)
    rng = np.random.default_rng(8)
    mpw = rng.uniform(0.1, 1.0, pos.shape[0]) * ion.spwt
    outs = []
    dom = GpuDomain(spec)
    try:
        dom.set_efield(efi, efj)
        km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=250000)
        km.set_weighted(True)
        km.set_sort_interval(2)
        km.add_particles(pos, vel, rewind=True, dt=1.25e-7, mpw=mpw)
        for _ in range(3):
            km.update_fields(1.25e-7)
        lc1, v1 = km.download()
        w1 = km.download_weights()
        km.sort()
        lc2, v2 = km.download()
        w2 = km.download_weights()
        a = np.lexsort(np.column_stack([lc1, v1, w1]).T)
        b = np.lexsort(np.column_stack([lc2, v2, w2]).T)
        assert np.array_equal(np.column_stack([lc1, v1, w1])[a], np.column_stack([lc2, v2, w2])[b])
        km.update_fields(1.25e-7)
        outs.append(km.get_count())
        # restart: the same particles and weights into a fresh context
        dom2 = GpuDomain(spec)
        try:
            dom2.set_efield(efi, efj)
            km2 = KineticMaterial(dom2, ion.mass, ion.charge, ion.spwt, capacity=250000)
            km2.set_weighted(True)
            km2.set_sort_interval(0)
            km2.add_particles_lc(lc2, v2, mpw=w2)
            km2.update_fields(1.25e-7)
            outs.append(km2.get_count())
        finally:
            dom2.close()
    finally:
        dom.close()
    assert np.array_equal(outs[0], outs[1])


def test_weighted_species_sources_emit_at_the_species_weight(gpulib):
    """A Maxwellian source on a weighted species gives the same particles and the same
    deposit as on a species of uniform weight (weight fraction 1)."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(81, 41, 1e-3)
    ion = W.IonSpecies()
    _, efi, efj = W.electrode_efield(spec)
    Ly = spec.lengths()[1]
    counts = []
    for weighted in (False, True):
        dom = GpuDomain(spec)
        try:
            dom.set_seed(3)
            dom.set_efield(efi, efj)
            km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=200000)
            km.set_weighted(weighted)
            for _ in range(3):
                km.sample_maxwellian_source([0.0, Ly, 0.0, 0.0], ion.den, ion.v_drift, ion.temp, 5e-7)
                km.update_fields(5e-7)
            counts.append(km.get_count())
            if weighted:
                assert np.all(km.download_weights() == ion.spwt)
        finally:
            dom.close()
    assert np.array_equal(counts[0], counts[1])


def _box():
    spec = W.es_pic_mesh(21, 21, 1e-3, walls=abi.DB_SYMMETRY, electrode_halfwidth=1e-12)
    spec.seg_xy = np.zeros((0, 4))
    spec.seg_btype = np.zeros(0, np.int32)
    spec.node_type[:] = abi.NODE_OPEN
    spec.bc_value[:] = 0
    return spec


def test_weighted_mcc_ionization_equals_a_species_of_that_weight(gpulib):
    """MCC ionization (MCC.java:167-221, 304-356) on a weighted species whose particles all
    carry half the species weight gives the collisions, products, S, count and weight sums of
    a uniform species of that half weight: S and the weight sum take each particle's mpw,
    the second electron the source electron's, the ion count spwt_src mpw/spwt / spwt_ion."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, MCC
    spec = _box()
    n, eV, e_ion = 100000, 50.0, 15.76
    me, mi, QE = 9.10938e-31, 40 * 1.66053886e-27, 1.60217646e-19
    spwt_e, spwt_i = 5e6, 1e6
    rng = np.random.default_rng(21)
    lc = rng.uniform(0.5, 19.5, (n, 2))
    lc = np.floor(lc) + (lc - np.floor(lc)).astype(np.float32).astype(np.float64)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    vel = (d * np.sqrt(2 * eV * QE / me)).astype(np.float32).astype(np.float64)
    nn = spec.nn
    den, T = np.full(nn, 1e20), np.full(nn, 300.0)
    out = []
    for weighted in (False, True):
        dom = GpuDomain(spec)
        try:
            dom.set_seed(4)
            dom.set_efield(np.zeros(nn), np.zeros(nn))
            ke = KineticMaterial(dom, me, -QE, spwt_e if weighted else 0.5 * spwt_e, capacity=2 * n)
            ki = KineticMaterial(dom, mi, QE, spwt_i, capacity=2 * n)
            if weighted:
                ke.set_weighted(True)
                ke.add_particles_lc(lc, vel, mpw=np.full(n, 0.5 * spwt_e))
            else:
                ke.add_particles_lc(lc, vel)
            mcc = MCC(dom, ke, target_mass=mi, den=den, temp=T, model=abi.MCC_IONIZATION,
                      sigma_model=abi.SIGMA_CONST, c=[1e-20, 0, 0, 0])
            cols, n_e, n_i = mcc.perform(5e-8, product=ki, ionization_energy=e_ion)
            sums = mcc.sums()
            _, evel = ke.download()
            w = ke.download_weights()
            out.append((cols, n_e, n_i, sums, evel, w))
        finally:
            dom.close()
    (c0, e0, i0, s0, v0, w0), (c1, e1, i1, s1, v1, w1) = out
    assert (c0, e0, i0) == (c1, e1, i1) and c0 > 0
    # the electrons collided in place are identical; the second electrons are appended in
    # atomic order, so the sets are compared
    assert np.array_equal(v0[:n], v1[:n])
    assert np.array_equal(v0[np.lexsort(v0.T)], v1[np.lexsort(v1.T)])
    assert np.allclose(w1, 0.5 * spwt_e) and np.allclose(w0, 0.5 * spwt_e)
    for key in ("S", "count_sum", "real_sum", "delta_n"):
        assert np.allclose(s0[key], s1[key], rtol=1e-12, atol=1e-12 * np.abs(s0[key]).max()), key


def test_weighted_dsmc_at_the_species_weight_equals_uniform(gpulib):
    """DSMC on a weighted species whose particles all carry the species weight collides as
    the uniform species (Boyd's update only acts on unequal weights, DSMC.java:431-452):
    the collision counts agree within their noise (the order the cell sort leaves inside a
    cell is set by atomics, so the pairs differ run to run), and the collided-weight sum is
    the count times the weight."""
    from starfish_gb300.plugin import DSMC, GpuDomain, KineticMaterial
    spec = _box()
    n, mass, spwt = 40000, 40 * 1.66053886e-27, 1e12
    rng = np.random.default_rng(6)
    lc = rng.uniform(0, 20, (n, 2))
    lc = np.floor(lc) + (lc - np.floor(lc)).astype(np.float32).astype(np.float64)
    vel = (rng.standard_normal((n, 3)) * 300.0).astype(np.float32).astype(np.float64)
    out = []
    for weighted in (False, True):
        dom = GpuDomain(spec)
        try:
            dom.set_seed(5)
            dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
            km = KineticMaterial(dom, mass, 0.0, spwt, capacity=n + 16)
            km.set_weighted(weighted)
            km.add_particles_lc(lc, vel, mpw=np.full(n, spwt) if weighted else None)
            ds = DSMC(dom, km, model=abi.SIGMA_BIRD463, diam=4.17e-10, T_ref=273.0, omega=0.81)
            cols = [ds.perform(1e-5) for _ in range(3)]
            cnt, real = ds.counts()
            _, v = km.download()
            out.append((cols, cnt, real, v))
        finally:
            dom.close()
    (c0, n0, r0, v0), (c1, n1, r1, v1) = out
    assert sum(c0) > 0
    assert abs(sum(c0) - sum(c1)) <= 5 * np.sqrt(sum(c0))
    assert np.allclose(r1, n1 * spwt, rtol=1e-12, atol=0)
    assert np.allclose(r0, n0 * spwt, rtol=1e-12, atol=0)
    assert n1.sum() == sum(c1)


def test_weight_rejections(gpulib):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(81, 41, 1e-3)
    ion = W.IonSpecies()
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=100)
        lc = np.array([[10.5, 10.5]])
        v = np.zeros((1, 3))
        # differing weights on a species of uniform weight
        with pytest.raises(abi.SfError):
            km.add_particles(lc * 1e-3, v, rewind=False, mpw=[0.5 * ion.spwt])
        km.set_weighted(True)
        # a weight above the species weight
        with pytest.raises(abi.SfError):
            km.add_particles_lc(lc, v, mpw=[2.0 * ion.spwt])
        km.add_particles_lc(lc, v, mpw=[0.5 * ion.spwt])
        # switching after the first particle
        with pytest.raises(abi.SfError):
            km.set_weighted(False)
    finally:
        dom.close()
