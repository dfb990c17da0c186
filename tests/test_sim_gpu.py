"""Whole-run check of the 81x41 ES-PIC case (tutorial-like: O+ beam from x = 0,
Boltzmann electrons, -100 V electrode): the GPU time loop (source, push + scatter,
rho, Poisson, E) against the oracle's loop over the same steps, four seeds each.  The
random streams differ (Philox on the GPU, java.util.Random in the oracle), so the
comparison is statistical: particle count, ion content and mean potential per run, and
the sampled moments of the last steps (KineticMaterial.updateSamples / computeFields,
KineticMaterial.java:1570-1671: density, mean velocity, temperature) over coarse
regions, within bounds set by the seed-to-seed spread of both codes."""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

EPS0 = 8.85418782e-12
QE = 1.60217646e-19
STEPS, SAMPLE_FROM = 60, 40
SEEDS = (0, 1, 2, 3)


def oracle_run(cfg, steps, seed=0, sample_from=SAMPLE_FROM):
    spec = cfg.mesh
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    ptr, idx = O.node_segments(m, spec.seg_xy)
    vol = O.node_volumes(m)
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_ABSORB)
    ion = cfg.ion
    Ly = spec.lengths()[1]
    inlet = np.array([0.0, Ly, 0.0, 0.0])
    phi = np.zeros(spec.nn)
    phi, _, _ = O.poisson_nl(m, spec.bc_value, np.zeros(spec.nn), cfg.n0, cfg.Te0, cfg.phi0, EPS0, phi,
                             max_it=20000, tol=1e-6, nl_max_it=50, nl_tol=1e-4)
    efi, efj = O.efield(m, phi)
    P = np.zeros((0, 12))
    rem = 0.0
    hist = []
    sums, ns = None, 0
    for it in range(steps):
        new, rem = O.maxwellian_source(seed * 100003 + it, inlet, ion.den, ion.v_drift, ion.temp, ion.mass,
                                       ion.spwt, cfg.dt, rem)
        O.add_particles(m, efi, efj, ion.charge, ion.mass, cfg.dt, new)
        P = np.ascontiguousarray(np.vstack([P, new]))
        O.push(m, efi, efj, ion.charge, ion.mass, cfg.dt, segs, ptr, idx, P, seed=seed * 7919 + it)
        P = np.ascontiguousarray(P[P[:, 10] == 1])
        den = O.update_fields(m, vol, P)
        if it >= sample_from:
            sums = O.update_samples(m, P, sums)
            ns += 1
        rho = QE * den
        phi, _, _ = O.poisson_nl(m, spec.bc_value, rho, cfg.n0, cfg.Te0, cfg.phi0, EPS0, phi,
                                 max_it=20000, tol=1e-6, nl_max_it=50, nl_tol=1e-4)
        efi, efj = O.efield(m, phi)
        hist.append((P.shape[0], (den * vol).sum(), phi.mean()))
    gas = O.compute_fields(sums, ns, vol, ion.mass, ion.temp)
    return np.array(hist), gas, phi


def gpu_run(cfg, steps, seed, sample_from=SAMPLE_FROM):
    from starfish_gb300.sim import EsPicSimulation
    sim = EsPicSimulation(cfg, seed=seed)
    try:
        hist = []
        sim.ions.clear_samples()
        for it in range(steps):
            st, sst = sim.step(sample=it >= sample_from)
            assert sst["status"] == 0
            den = sim.ions.get_den()
            vol = sim.dom.get_field(5)
            phi = sim.dom.get_field(10)
            hist.append((st["np"], (den * vol).sum(), phi.mean()))
        gas = sim.ions.compute_fields(cfg.ion.temp)
        phi = sim.dom.get_field(10)
    finally:
        sim.close()
    return np.array(hist), gas, phi


def _blocks(f, spec, b=8):
    """Means over b x b node blocks (the last node row and column dropped)."""
    a = f.reshape(spec.nj, spec.ni)[:spec.nj - 1, :spec.ni - 1]
    nj, ni = (spec.nj - 1) // b, (spec.ni - 1) // b
    return a[:nj * b, :ni * b].reshape(nj, b, ni, b).mean(axis=(1, 3))


def _agree(g, o, mask, rel, k=4.0):
    """Seed means agree within k standard errors of the difference plus rel of |oracle|."""
    gm, om = g.mean(axis=0), o.mean(axis=0)
    se = np.sqrt(g.var(axis=0, ddof=1) / g.shape[0] + o.var(axis=0, ddof=1) / o.shape[0])
    bad = mask & (np.abs(gm - om) > k * se + rel * np.abs(om))
    return int(bad.sum()), gm[mask], om[mask]


def test_es_pic_81x41_whole_run_over_seeds(gpulib):
    cfg = W.config0()
    spec = cfg.mesh
    g = [gpu_run(cfg, STEPS, s) for s in SEEDS]
    o = [oracle_run(cfg, STEPS, s) for s in SEEDS]
    for h, _, phi in g:
        assert np.all(np.isfinite(h))
        # the electrode and walls hold their potential
        assert phi.min() == pytest.approx(-100.0, abs=1e-6)
    # particle count, ion content and mean potential over the last 20 steps of each run
    gh = np.array([h[-20:].mean(axis=0) for h, _, _ in g])
    oh = np.array([h[-20:].mean(axis=0) for h, _, _ in o])
    ok = np.array([True, True, True])
    nbad, gm, om = _agree(gh, oh, ok, np.array([0.02, 0.02, 0.02]))
    assert nbad == 0, (gm, om)
    # sampled moments of the last 20 steps over 8x8-node blocks
    nd_g = np.array([_blocks(x[1]["nd-ave"], spec) for x in g])
    nd_o = np.array([_blocks(x[1]["nd-ave"], spec) for x in o])
    dense = nd_o.mean(axis=0) > 0.1 * nd_o.mean(axis=0).max()
    assert dense.sum() >= 10
    nbad, gm, om = _agree(nd_g, nd_o, dense, 0.03)
    assert nbad == 0, ("nd", gm, om)
    for key, rel in (("u-ave", 0.02), ("v-ave", 0.0), ("T", 0.03)):
        fg = np.array([_blocks(x[1][key], spec) for x in g])
        fo = np.array([_blocks(x[1][key], spec) for x in o])
        if key == "v-ave":
            # the mean v is near zero: compare against the thermal speed scale instead
            scale = np.sqrt(1.3806503e-23 * cfg.ion.temp / cfg.ion.mass)
            gm_, om_ = fg.mean(axis=0), fo.mean(axis=0)
            se = np.sqrt(fg.var(axis=0, ddof=1) / len(SEEDS) + fo.var(axis=0, ddof=1) / len(SEEDS))
            bad = dense & (np.abs(gm_ - om_) > 4 * se + 0.02 * scale)
            assert bad.sum() == 0, (key, gm_[dense], om_[dense])
            continue
        nbad, gm, om = _agree(fg, fo, dense, rel)
        assert nbad == 0, (key, gm, om)
