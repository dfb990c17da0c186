"""Axisymmetric (ZR) push and scatter against the oracle: rotateToZR
(KineticMaterial.java:444-462), the Ruyten radial weights of Field2D.scatter
(Field2D.java:254-285), the symmetry axis and diffuse walls (SurfaceInteraction.java:153-213)."""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

KB = 1.3806503e-23


def small_jet():
    return W.jet_mesh(ni=65, nj=33, Lz=0.064, Lr=0.032, r_inlet=4e-3)


def state(spec, n, seed, speed=400.0):
    rng = np.random.default_rng(seed)
    lc = np.column_stack([rng.uniform(0, spec.ni - 1.001, n), rng.uniform(0, spec.nj - 1.001, n)])
    i = np.floor(lc)
    lc = i + (lc - i).astype(np.float32).astype(np.float64)
    vel = (rng.standard_normal((n, 3)) * speed).astype(np.float32).astype(np.float64)
    return lc, vel


def oracle_parts(spec, lc, vel, w):
    P = np.zeros((lc.shape[0], 12))
    P[:, 0] = spec.x0[0] + lc[:, 0] * spec.dh[0]
    P[:, 1] = spec.x0[1] + lc[:, 1] * spec.dh[1]
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = w
    P[:, 10] = 1
    return P


def gpu_push(spec, lc, vel, mass, w, dt, vth):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    dom = GpuDomain(spec)
    dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
    km = KineticMaterial(dom, mass, 0.0, w, capacity=lc.shape[0] + 16)
    for s in range(spec.seg_xy.shape[0]):
        km.set_surface(s, abi.SURF_DIFFUSE, vth=vth, c_rest=1.0, c_accom=1.0)
    km.set_sort_interval(0)
    km.add_particles_lc(lc, vel)
    st = km.update_fields(dt)
    glc, gvel = km.download()
    den = km.get_den()
    flux, _ = km.surface_flux()
    dom.close()
    return glc, gvel, den, flux, st


def test_zr_scatter_ruyten_weights(gpulib):
    spec = small_jet()
    mass, w = 40 * 1.66053886e-27, 1e10
    lc, vel = state(spec, 20000, 1)
    glc, gvel, den, flux, st = gpu_push(spec, lc, vel, mass, w, 1e-15, 300.0)
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    vol = O.node_volumes(m)
    P = oracle_parts(spec, lc, vel, w)
    oden = O.update_fields(m, vol, P)
    # node volumes of the axisymmetric mesh agree with the oracle's Mesh.nodeVol
    from starfish_gb300.plugin import GpuDomain
    d = GpuDomain(spec)
    gvol = d.get_field(abi.FIELD_NODE_VOL)
    d.close()
    assert np.allclose(gvol, vol, rtol=1e-12)
    assert np.max(np.abs(den - oden)) <= 1e-6 * np.abs(oden).max()


def test_zr_push_with_diffuse_walls(gpulib):
    spec = small_jet()
    mass, w = 40 * 1.66053886e-27, 1e10
    vth = np.sqrt(2 * KB * 300.0 / mass)
    lc, vel = state(spec, 40000, 2, speed=600.0)
    dt = 2e-6
    glc, gvel, den, gflux, st = gpu_push(spec, lc, vel, mass, w, dt, vth)
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    ptr, idx = O.node_segments(m, spec.seg_xy)
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_DIFFUSE, vth=vth, c_rest=1.0, c_accom=1.0)
    P = oracle_parts(spec, lc, vel, w)
    speed0 = np.linalg.norm(vel, axis=1)
    alive, ost, oflux, _ = O.push(m, np.zeros(spec.nn), np.zeros(spec.nn), 0.0, mass, dt, segs, ptr, idx, P, seed=3)
    keep = P[:, 10] == 1
    assert glc.shape[0] == keep.sum()
    # particles that met no wall keep their speed (the ZR rotation is a rotation): exact match
    speed1 = np.linalg.norm(P[:, 3:6], axis=1)
    plain = np.abs(speed1 - speed0) <= 1e-9 * speed0
    sel = plain[keep]
    assert sel.sum() > 0.9 * keep.sum()
    assert np.max(np.abs(glc[sel] - P[keep][sel, 6:8])) < 1e-5
    assert np.max(np.abs(gvel[sel] - P[keep][sel, 3:6]) / speed0[keep][sel, None]) < 1e-5
    # wall hits are decided before any random re-emission: the first-hit flux agrees
    assert gflux.sum() == pytest.approx(oflux.sum(), rel=0.02)
    # diffusely re-emitted particles carry the wall temperature: mean speed ~ 2 vth / sqrt(pi)
    hit = ~plain[keep]
    gspeed = np.linalg.norm(gvel, axis=1)
    assert hit.sum() > 100
    assert gspeed[hit].mean() == pytest.approx(2 * vth / np.sqrt(np.pi), rel=0.1)


def test_zr_source_area_weighted(gpulib):
    """Device Maxwellian source on the axisymmetric jet mesh: the particle count uses the
    frustum area pi (r1 + r2) L, and positions are uniform in the swept area (Spline.randomT
    on RZ/ZR meshes), so on the inlet r in [0, R] the radius has density 2 r / R^2."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.jet_mesh()
    R, mass, spwt = 5e-3, 40 * 1.66053886e-27, 1e9
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, mass, 0.0, spwt, capacity=1 << 20)
        n = km.sample_maxwellian_source(np.array([0.0, R, 0.0, 0.0]), 1e22, 500.0, 300.0, 1e-6)
        v_mean = np.sqrt(8 * 1.3806503e-23 * 300.0 / (np.pi * mass))
        assert n == int(1e22 * np.pi * R * R * (500.0 + v_mean / 4) * 1e-6 / spwt)
        lc, vel = km.download()
        r = lc[:, 1] * spec.dh[1]
        assert np.mean(r) == pytest.approx(2 * R / 3, rel=5e-3)
        assert np.median(r) == pytest.approx(R / np.sqrt(2), rel=5e-3)
        assert np.all(vel[:, 0] > 0)  # v . n > 0 on the inlet (normal +z)
    finally:
        dom.close()
