"""The nonlinear Poisson solve on axisymmetric meshes (RZ: radius along i, ZR: radius
along j) against the oracle: the reference's FVM operator with face fluxes weighted by
the face radius over the node volume 2 pi r dA (Solver.java:451-553, Mesh.nodeVol
Mesh.java:998-1020), a symmetry face on the axis, Dirichlet outer walls and a ring
electrode.  The GPU potential must satisfy the oracle's assembled operator and agree
with the oracle's own NR + SOR solution."""
import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

EPS0 = 8.85418782e-12
QE = 1.60217646e-19


def axi_mesh(domain, ni=65, nj=33, dh=1e-3, r0=0.0):
    """es_pic_mesh turned axisymmetric: the axis face (bottom for ZR, left for RZ) is a
    symmetry face with open nodes when r0 = 0; the electrode becomes a ring."""
    spec = W.es_pic_mesh(ni, nj, dh, electrode_halfwidth=4e-3)
    spec.domain = domain
    nt = spec.node_type.reshape(nj, ni)
    if domain == abi.DOMAIN_ZR:
        spec.x0 = (0.0, r0)
        if r0 == 0.0:
            spec.face_type[abi.FACE_BOTTOM, :] = abi.DB_SYMMETRY
            nt[0, 1:-1] = abi.NODE_OPEN
    else:
        spec.x0 = (r0, 0.0)
        if r0 == 0.0:
            spec.face_type[abi.FACE_LEFT, :] = abi.DB_SYMMETRY
            nt[1:-1, 0] = abi.NODE_OPEN
    spec.node_type = nt.reshape(-1)
    spec.seg_xy = spec.seg_xy + np.array([spec.x0[0], spec.x0[1], spec.x0[0], spec.x0[1]])
    spec.node_seg_ptr = spec.node_seg_idx = None
    return spec


def ion_rho(spec, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, spec.ni)
    y = np.linspace(0, 1, spec.nj)
    X, Y = np.meshgrid(x, y)
    n = 1e12 * (0.6 + 0.4 * np.cos(2 * np.pi * X) * np.sin(np.pi * Y)) * (1 + 0.05 * rng.standard_normal(X.shape))
    n = n.reshape(-1)
    n[spec.node_type == abi.NODE_DIRICHLET] = 0
    return QE * n


@pytest.mark.parametrize("domain,r0", [(abi.DOMAIN_ZR, 0.0), (abi.DOMAIN_RZ, 0.0), (abi.DOMAIN_ZR, 5e-3)])
def test_axisymmetric_poisson_matches_oracle(gpulib, domain, r0):
    from starfish_gb300.plugin import GpuDomain, PoissonSolver
    spec = axi_mesh(domain, r0=r0)
    rho = ion_rho(spec, 3)
    dom = GpuDomain(spec)
    try:
        ps = PoissonSolver(dom, n0=1e12, Te0=2.0, phi0=0.0, tol=1e-9, max_it=80)
        phi_g, st = ps.solve(rho=rho, phi=np.zeros(spec.nn))
        efi, efj = ps.update_gradient_field(copy=True)
    finally:
        dom.close()
    assert st["residual"] < 1e-9
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    # the GPU potential satisfies the reference's assembled axisymmetric operator
    r = O.poisson_residual(m, spec.bc_value, rho, 1e12, 2.0, 0.0, EPS0, phi_g)
    assert r / spec.nn < 1e-8, r / spec.nn
    # and agrees with the oracle's own solution (NR + SOR driven to its floor)
    phi_o, _, _ = O.poisson_nl(m, spec.bc_value, rho, 1e12, 2.0, 0.0, EPS0, np.zeros(spec.nn),
                               max_it=200000, tol=1e-10, nl_max_it=60, nl_tol=1e-9)
    assert np.max(np.abs(phi_g - phi_o)) < 1e-6
    assert phi_g.min() == pytest.approx(-100.0, abs=1e-9)
    # E = -grad(phi) as the oracle evaluates it
    oi, oj = O.efield(m, phi_g)
    scale = np.abs(oi).max() + np.abs(oj).max()
    assert np.max(np.abs(efi - oi)) <= 1e-12 * scale + 1e-9
    assert np.max(np.abs(efj - oj)) <= 1e-12 * scale + 1e-9


def test_axisymmetric_rejects_learned_modes(gpulib):
    from starfish_gb300.plugin import GpuDomain, PoissonSolver
    spec = axi_mesh(abi.DOMAIN_ZR)
    dom = GpuDomain(spec)
    try:
        ps = PoissonSolver(dom, n0=1e12, Te0=2.0, phi0=0.0, tol=1e-6, max_it=40)
        ps.use_learned(True, 1)
        with pytest.raises(abi.SfError):
            ps.solve(rho=ion_rho(spec, 1), phi=np.zeros(spec.nn))
    finally:
        dom.close()
