"""Whole-run check of the 81x41 ES-PIC case (tutorial-like: O+ beam from x = 0,
Boltzmann electrons, -100 V electrode): the GPU time loop (source, push + scatter,
rho, Poisson, E) against the oracle's loop over the same steps.  The random streams
differ (Philox on the GPU, java.util.Random in the oracle), so the comparison is of
whole-run moments: particle count, total ion content, mean density, potential."""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

EPS0 = 8.85418782e-12
QE = 1.60217646e-19


def oracle_run(cfg, steps, seed=0):
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
    for it in range(steps):
        new, rem = O.maxwellian_source(seed * 100003 + it, inlet, ion.den, ion.v_drift, ion.temp, ion.mass,
                                       ion.spwt, cfg.dt, rem)
        O.add_particles(m, efi, efj, ion.charge, ion.mass, cfg.dt, new)
        P = np.ascontiguousarray(np.vstack([P, new]))
        O.push(m, efi, efj, ion.charge, ion.mass, cfg.dt, segs, ptr, idx, P, seed=it)
        P = np.ascontiguousarray(P[P[:, 10] == 1])
        den = O.update_fields(m, vol, P)
        rho = QE * den
        phi, _, _ = O.poisson_nl(m, spec.bc_value, rho, cfg.n0, cfg.Te0, cfg.phi0, EPS0, phi,
                                 max_it=20000, tol=1e-6, nl_max_it=50, nl_tol=1e-4)
        efi, efj = O.efield(m, phi)
        hist.append((P.shape[0], (den * vol).sum(), phi.mean()))
    return np.array(hist), den, phi


def test_es_pic_81x41_whole_run(gpulib):
    from starfish_gb300.sim import EsPicSimulation
    cfg = W.config0()
    steps = 60
    sim = EsPicSimulation(cfg)
    ghist = []
    for _ in range(steps):
        st, sst = sim.step()
        assert sst["status"] == 0
        den = sim.ions.get_den()
        vol = sim.dom.get_field(5)
        phi = sim.dom.get_field(10)
        ghist.append((st["np"], (den * vol).sum(), phi.mean()))
    gden = sim.ions.get_den()
    gphi = sim.dom.get_field(10)
    sim.close()
    ghist = np.array(ghist)
    ohist, oden, ophi = oracle_run(cfg, steps)
    assert np.all(np.isfinite(ghist))
    # particle count and ion content over the last 20 steps within a few percent
    g = ghist[-20:].mean(axis=0)
    o = ohist[-20:].mean(axis=0)
    assert g[0] == pytest.approx(o[0], rel=0.05)
    assert g[1] == pytest.approx(o[1], rel=0.05)
    # the electrode and walls hold their potential; the mean potential agrees
    assert gphi.min() == pytest.approx(-100.0, abs=1e-6)
    assert g[2] == pytest.approx(o[2], rel=0.05, abs=0.5)
