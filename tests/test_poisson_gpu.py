"""GPU parity of the nonlinear Poisson solve, the electric field and the Boltzmann
electrons against the oracle (PoissonSolver.update + Solver.solveNonLinearNR with the
serial GS solver, the assembled FVM operator, Solver.evaluateGradient).

The converged potentials are compared after both solvers were driven well below the
tolerance used in production; the GPU solution's residual is also evaluated with the
oracle's own assembled matrix.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

EPS0 = 8.85418782e-12
QE = 1.60217646e-19


def _omesh(spec):
    return O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)


def ion_rho(spec, seed, n_mean=1e12):
    """A smooth-plus-noise ion charge density (C/m^3), zero inside the electrode."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, spec.ni)
    y = np.linspace(0, 1, spec.nj)
    X, Y = np.meshgrid(x, y)
    n = n_mean * (0.6 + 0.4 * np.cos(2 * np.pi * X) * np.sin(np.pi * Y)) * (1 + 0.05 * rng.standard_normal(X.shape))
    n = n.reshape(-1)
    n[spec.node_type == abi.NODE_DIRICHLET] = 0
    return QE * n


def gpu_solve(spec, rho, tol, phi_init=None, linear=False, max_it=80):
    from starfish_gb300.plugin import GpuDomain, PoissonSolver
    dom = GpuDomain(spec)
    ps = PoissonSolver(dom, n0=1e12, Te0=2.0, phi0=0.0, tol=tol, max_it=max_it, linear=linear)
    phi0 = np.zeros(spec.nn) if phi_init is None else phi_init
    phi, st = ps.solve(rho=rho, phi=phi0)
    efi, efj = ps.update_gradient_field(copy=True)
    ne = None if linear else ps.boltzmann()
    dom.close()
    return phi, st, efi, efj, ne


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_poisson_nl_matches_oracle_c0(gpulib):
    """Golden fixture: the oracle's NR+GS solution driven to its FP64 floor
    (||R||_2/N ~ 2e-10 on this mesh; tests/golden/make_golden.py)."""
    spec = W.es_pic_mesh(81, 41, 1e-3)
    g = np.load(os.path.join(GOLDEN, "poisson_es_pic_81x41.npz"))
    rho, phi_o = g["rho"], g["phi"]
    m = _omesh(spec)
    phi_g, st, efi, efj, ne = gpu_solve(spec, rho, tol=5e-10)
    assert st["residual"] < 5e-10
    # the two converged potentials agree far below the volt scale of the problem (100 V)
    assert np.max(np.abs(phi_g - phi_o)) < 1e-7
    # the GPU potential satisfies the oracle's assembled operator
    # (the operators differ only in FP64 rounding of their coefficients, ~1e-16 relative)
    r = O.poisson_residual(m, spec.bc_value, rho, 1e12, 2.0, 0.0, EPS0, phi_g)
    assert r / spec.nn < 1e-8
    # E = -grad(phi) and the Boltzmann density
    oi, oj = O.efield(m, phi_g)
    scale = np.abs(oi).max() + np.abs(oj).max()
    assert np.max(np.abs(efi - oi)) <= 1e-12 * scale + 1e-9
    assert np.max(np.abs(efj - oj)) <= 1e-12 * scale + 1e-9
    one = O.boltzmann(phi_g, 1e12, 2.0, 0.0)
    assert np.allclose(ne, one, rtol=1e-12)


def test_poisson_production_tolerance(gpulib):
    """At the production tolerance (1e-6 on ||R||_2/N) the potential already matches the
    tightly converged oracle solution to well under a millivolt."""
    spec = W.es_pic_mesh(81, 41, 1e-3)
    g = np.load(os.path.join(GOLDEN, "poisson_es_pic_81x41.npz"))
    rho, phi_o = g["rho"], g["phi"]
    phi_g, st, _, _, _ = gpu_solve(spec, rho, tol=1e-6)
    assert st["residual"] < 1e-6
    assert np.max(np.abs(phi_g - phi_o)) < 1e-3


def test_poisson_linear_neumann_faces(gpulib):
    """Linear mode with Dirichlet left/right walls and open (Neumann) top/bottom faces:
    the discrete solution with rho = 0 is linear in x."""
    ni, nj, dh = 129, 65, 1e-3
    spec = W.es_pic_mesh(ni, nj, dh, walls=abi.DB_DIRICHLET, electrode_halfwidth=1e-9)
    spec.seg_xy = np.zeros((0, 4))
    spec.seg_btype = np.zeros(0, np.int32)
    nt = np.full((nj, ni), abi.NODE_OPEN, np.int8)
    nt[:, 0] = nt[:, -1] = abi.NODE_DIRICHLET
    spec.node_type = nt.reshape(-1)
    spec.face_type[abi.FACE_TOP, :] = abi.DB_SYMMETRY
    spec.face_type[abi.FACE_BOTTOM, :] = abi.DB_SYMMETRY
    bc = np.zeros((nj, ni))
    bc[:, 0] = 10.0
    spec.bc_value = bc.reshape(-1)
    phi_g, st, _, _, _ = gpu_solve(spec, np.zeros(spec.nn), tol=1e-10, linear=True)
    exact = np.tile(10.0 * (1.0 - np.arange(ni) / (ni - 1)), nj)
    assert np.max(np.abs(phi_g - exact)) < 1e-8


def test_poisson_large_mesh_residual(gpulib):
    """2049x1025 (the scaled workload): reach 1e-6 from a cold start; the residual is
    re-evaluated in FP64 with numpy from the returned potential."""
    spec = W.es_pic_mesh(2049, 1025, 5e-5, electrode_halfwidth=4.5e-3)
    rho = ion_rho(spec, 7)
    phi, st, efi, efj, ne = gpu_solve(spec, rho, tol=1e-6, max_it=100)
    assert st["residual"] < 1e-6
    ni, nj = spec.ni, spec.nj
    P = phi.reshape(nj, ni)
    dx = spec.dh[0]
    fixed = (spec.node_type != abi.NODE_OPEN).reshape(nj, ni)
    lap = np.zeros_like(P)
    lap[1:-1, 1:-1] = (P[1:-1, 2:] + P[1:-1, :-2] - 2 * P[1:-1, 1:-1]) / dx**2 + \
                      (P[2:, 1:-1] + P[:-2, 1:-1] - 2 * P[1:-1, 1:-1]) / dx**2
    R = lap - (-rho.reshape(nj, ni) / EPS0 + QE / EPS0 * 1e12 * np.exp(P / 2.0))
    R[fixed] = (P - spec.bc_value.reshape(nj, ni))[fixed]
    assert np.sqrt((R ** 2).sum()) / spec.nn < 1e-6


def test_solves_independent_of_other_contexts(gpulib):
    """Two contexts in one process: A (81x41, large single-CTA coarse end), then B
    (33x17, small coarse end), then A solves again with another PCG iteration count, so
    its Newton step is captured anew after B was set up.  Each context's result must not
    depend on the other's existence: A's potential equals that of A alone, bit for bit."""
    from starfish_gb300.plugin import GpuDomain, PoissonSolver
    big, small = W.es_pic_mesh(81, 41, 1e-3), W.es_pic_mesh(33, 17, 1e-3)
    rho_b, rho_s = ion_rho(big, 1), ion_rho(small, 2)

    def solve(dom, spec, rho, cycles):
        ps = PoissonSolver(dom, n0=1e12, Te0=2.0, tol=1e-6, max_it=60, cycles=cycles)
        return ps.solve(rho=rho, phi=np.zeros(spec.nn))

    alone = GpuDomain(big)
    try:
        ref4, _ = solve(alone, big, rho_b, 4)
        ref3, _ = solve(alone, big, rho_b, 3)
    finally:
        alone.close()
    a, b = GpuDomain(big), GpuDomain(small)
    try:
        p4, _ = solve(a, big, rho_b, 4)
        _, sb = solve(b, small, rho_s, 4)
        p3, st = solve(a, big, rho_b, 3)
        assert sb["status"] == 0 and st["status"] == 0
        assert np.array_equal(p4, ref4) and np.array_equal(p3, ref3)
    finally:
        a.close()
        b.close()


def test_failures_reported_and_context_usable(gpulib):
    """Failure detection without a GPU fault: a NaN in rho gives SF_ERR_DIVERGED, too few
    Newton steps SF_ERR_NOT_CONVERGED (the Java caller then falls back to its own solver);
    either way the context solves normally afterwards."""
    from starfish_gb300.plugin import GpuDomain, PoissonSolver
    spec = W.es_pic_mesh(81, 41, 1e-3)
    rho = ion_rho(spec, 4)
    dom = GpuDomain(spec)
    try:
        bad = rho.copy()
        bad[spec.nn // 2 + 10] = np.nan
        _, st = PoissonSolver(dom, tol=1e-6, max_it=60).solve(rho=bad, phi=np.zeros(spec.nn), check=False)
        assert st["status"] == abi.SF_ERR_DIVERGED
        _, st = PoissonSolver(dom, tol=1e-6, max_it=1).solve(rho=rho, phi=np.zeros(spec.nn), check=False)
        assert st["status"] == abi.SF_ERR_NOT_CONVERGED and st["newton_it"] == 1
        phi, st = PoissonSolver(dom, tol=1e-6, max_it=60).solve(rho=rho, phi=np.zeros(spec.nn))
        assert st["status"] == 0 and st["residual"] < 1e-6 and np.all(np.isfinite(phi))
    finally:
        dom.close()


def test_batch_failure_names_instance_and_batch_recovers(gpulib):
    """A batched solve that cannot converge in its Newton budget fails the step with the
    instance named; the batch then steps normally with a sufficient budget."""
    from starfish_gb300.plugin import GpuBatch, GpuDomain, KineticMaterial, PoissonSolver
    cases = W.config4(3, seed=5, max_particles=20_000, min_particles=10_000)
    doms, kms, sol = [], [], []
    for c in cases:
        d = GpuDomain(c.mesh)
        ps = PoissonSolver(d, n0=1e12, Te0=2.0, tol=1e-6, max_it=60)
        ps.solve(rho=np.zeros(c.mesh.nn), phi=np.zeros(c.mesh.nn))
        ps.update_gradient_field()
        km = KineticMaterial(d, c.ion.mass, c.ion.charge, c.ion.spwt, capacity=3 * c.n_particles)
        pos, vel = W.uniform_maxwellian(c.mesh, c.ion, c.n_particles, c.seed)
        km.add_particles(pos, vel, rewind=True, dt=5e-7)
        doms.append(d)
        kms.append(km)
        sol.append(ps)
    batch = GpuBatch(doms, kms, threads=2)
    try:
        strict = PoissonSolver(doms[0], n0=1e12, Te0=2.0, tol=1e-14, max_it=2)
        with pytest.raises(abi.SfError) as e:
            batch.step(5e-7, strict)
        assert e.value.code == abi.SF_ERR_NOT_CONVERGED and "instance" in str(e.value)
        st = batch.step(5e-7, sol[0])
        assert st["particles"] > 0
    finally:
        batch.close()
        for d in doms:
            d.close()
