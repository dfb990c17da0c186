"""Batches of independent instances (sf_batch_*) against the per-instance entry points.

Each instance has a twin context with the same mesh, particles and field.  One batch
step (batched push + scatter, then each instance's rho, Poisson solve and E) must give
what the twin gets from sf_push_deposit, sf_update_rho, sf_poisson_nl and sf_efield:
the deposit is integer fixed point and the solve is deterministic, so densities and
potentials agree exactly and the particle sets are equal.  The batched source is checked
for its count and placement; the autotuner for settling on a launch shape and on the PCG
iterations per mesh-size bucket.
"""
import numpy as np
import pytest

from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _instance(case, dt, weighted=False):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, PoissonSolver
    spec, ion = case.mesh, case.ion
    dom = GpuDomain(spec)
    ps = PoissonSolver(dom, n0=1e12, Te0=2.0, tol=1e-6, max_it=60, cycles=2)
    ps.solve(rho=np.zeros(spec.nn), phi=np.zeros(spec.nn))
    ps.update_gradient_field()
    # removed slots stay until the next sort (every 16 steps) while the inlet keeps adding
    km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt, capacity=int(case.n_particles * 3) + 8192)
    pos, vel = W.uniform_maxwellian(spec, ion, case.n_particles, case.seed)
    mpw = None
    if weighted:
        km.set_weighted(True)
        mpw = ion.spwt * np.random.default_rng(case.seed + 77).uniform(0.2, 1.0, case.n_particles)
    km.add_particles(pos, vel, rewind=True, dt=dt, mpw=mpw)
    return dom, km, ps


def _sorted(lc, vel):
    a = np.hstack([lc, vel])
    return a[np.lexsort(a.T[::-1])]


def _batch_vs_twins(cases, dt, threads, weighted=()):
    from starfish_gb300.plugin import GpuBatch
    A = [_instance(c, dt, k in weighted) for k, c in enumerate(cases)]
    B = [_instance(c, dt, k in weighted) for k, c in enumerate(cases)]
    batch = GpuBatch([a[0] for a in A], [a[1] for a in A], threads=threads)
    try:
        st = batch.step(dt, A[0][2])  # first step: PCG iterations 2 in every bucket (tuning)
        assert st["particles"] > 0 and st["capacity_overflow"] == 0
        for (da, ka, pa), (db, kb, pb) in zip(A, B):
            kb.update_fields(dt, stats=False)
            pb.update_rho()
            pb.prm.cycles = 2
            pb.solve()
            pb.update_gradient_field()
            assert np.array_equal(ka.get_den(), kb.get_den())
            assert np.array_equal(da.get_field(abi.FIELD_PHI), db.get_field(abi.FIELD_PHI))
            assert np.array_equal(da.get_field(abi.FIELD_EFI), db.get_field(abi.FIELD_EFI))
            assert ka.get_np() == kb.get_np()
            assert np.array_equal(_sorted(*ka.download()), _sorted(*kb.download()))
            if weighted:
                la, va = ka.download()
                lb, vb = kb.download()
                wa, wb = ka.download_weights(), kb.download_weights()
                assert np.array_equal(_sorted(la, np.column_stack([va, wa])), _sorted(lb, np.column_stack([vb, wb])))
        live = sum(a[1].get_np() for a in A)
        assert st["particles"] == live
    finally:
        batch.close()
        for d in A + B:
            d[0].close()


def test_batch_step_matches_instances(gpulib):
    _batch_vs_twins(W.config4(6, seed=3, max_particles=200_000, min_particles=20_000), 5e-7, 3)


def test_batch_with_weighted_species_matches_instances(gpulib):
    """Instances 0 and 3 carry per-particle weights (mpw uniform in [0.2, 1] spwt), the
    others uniform weight: the batched push deposits each particle's weight, as the
    per-instance push does, bit for bit."""
    _batch_vs_twins(W.config4(5, seed=8, max_particles=150_000, min_particles=20_000), 5e-7, 2, weighted=(0, 3))


def test_batch_solve_matches_tiled_levels_on_a_large_mesh(gpulib):
    """A 2049x513 instance (over 2^20 nodes: the per-instance solve runs its finest level
    on 64x16 tiles and the next ones on 32x8 tiles) against the batched solve's global
    red-black sweeps: the same values bit for bit."""
    m = W.es_pic_mesh(2049, 513, 1e-4, electrode_halfwidth=4.5e-3, phi_electrode=-150.0)
    n = 50_000
    Lx, Ly = m.lengths()
    ion = W.IonSpecies(spwt=1e12 * (Lx * Ly - (2 * 4.5e-3) ** 2) / n)
    _batch_vs_twins([W.BatchCase(m, ion, n, -150.0, 0)], 2e-7, 1)


def test_batch_source_and_tuning(gpulib):
    from starfish_gb300.plugin import GpuBatch
    dt = 5e-7
    cases = W.config4(4, seed=11, max_particles=50_000, min_particles=10_000)
    A = [_instance(c, dt) for c in cases]
    B = [_instance(c, dt) for c in cases]
    ion = cases[0].ion
    batch = GpuBatch([a[0] for a in A], [a[1] for a in A], threads=2)
    try:
        for i, c in enumerate(cases):
            Lx, Ly = c.mesh.lengths()
            batch.set_source(i, [0.0, Ly, 0.0, 0.0], ion.den, ion.v_drift, ion.temp)
        batch.step(dt, A[0][2])
        for i, c in enumerate(cases):
            Lx, Ly = c.mesh.lengths()
            km = B[i][1]
            added = km.sample_maxwellian_source(np.array([0.0, Ly, 0.0, 0.0]), ion.den, ion.v_drift, ion.temp, dt)
            assert added > 0
            km.update_fields(dt, stats=False)
            # same number injected (the positions come from different random streams),
            # so the live counts agree up to the few particles that differ in removal
            assert abs(A[i][1].get_np() - km.get_np()) <= max(2, added // 200)
            # the injected particles sit near the inlet in both after one push
            near_a = int(np.sum(A[i][1].download()[0][:, 0] < 6.0))
            near_b = int(np.sum(km.download()[0][:, 0] < 6.0))
            assert abs(near_a - near_b) <= max(5, added // 50), (near_a, near_b, added)
        for _ in range(12):
            st = batch.step(dt, A[0][2])
            assert st["capacity_overflow"] == 0
        t = batch.tuning()
        assert t["push_blocks_per_sm"] in (1, 2, 4) and t["slow_blocks_per_sm"] in (8, 16)
        buckets = {0 if c.mesh.nn < 4096 else (1 if c.mesh.nn < 16384 else 2) for c in cases}
        for k in buckets:
            assert t["pcg_iterations_by_bucket"][k] in (2, 3, 4)
    finally:
        batch.close()
        for d in A + B:
            d[0].close()
