"""Time loop of an ES-PIC case on the GPU, in the order of Starfish.MainLoop
(core/common/Starfish.java:67-126): sources -> materials (push + scatter, Boltzmann
electrons) -> field solve (rho, Poisson, E).  The state stays on the device; the host
only sequences the C-ABI calls.
"""
from __future__ import annotations

import time

import numpy as np

from . import workloads as W
from .plugin import GpuDomain, KineticMaterial, PoissonSolver


class EsPicSimulation:
    def __init__(self, cfg: W.EsPicConfig, device=0, capacity=None, inlet=True, seed_particles=None,
                 poisson_tol=1e-6, seed=None):
        self.cfg = cfg
        self.dom = GpuDomain(cfg.mesh, device=device)
        if seed is not None:
            self.dom.set_seed(seed)
        ion = cfg.ion
        cap = capacity or max(4 * cfg.n_particles, 1 << 20)
        self.ions = KineticMaterial(self.dom, ion.mass, ion.charge, ion.spwt, capacity=cap)
        self.solver = PoissonSolver(self.dom, n0=cfg.n0, Te0=cfg.Te0, phi0=cfg.phi0, tol=poisson_tol,
                                    max_it=60, cycles=4)
        Lx, Ly = cfg.mesh.lengths()
        x0, y0 = cfg.mesh.x0
        # inlet on the x = x0 face, drifting into +x: segment from top to bottom so that the
        # LinearSegment normal (-dy, dx)/L points along +x
        self.inlet = np.array([x0, y0 + Ly, x0, y0]) if inlet else None
        self.it = 0
        self.timings = {"source": 0.0, "push": 0.0, "solve": 0.0}
        self.solve_stats = []
        # initial field: solve with no charge, then E
        self.solver.solve(rho=np.zeros(cfg.mesh.nn), phi=np.zeros(cfg.mesh.nn))
        self.solver.update_gradient_field()
        if seed_particles is not None:
            pos, vel = seed_particles
            self.ions.add_particles(pos, vel, rewind=True, dt=cfg.dt)

    def step(self, sample=False):
        """One time step; sample=True also adds the ions to the velocity samples
        (KineticMaterial.updateSamples, after clear_samples)."""
        cfg = self.cfg
        t0 = time.perf_counter()
        if self.inlet is not None:
            self.ions.sample_maxwellian_source(self.inlet, cfg.ion.den, cfg.ion.v_drift, cfg.ion.temp, cfg.dt)
        t1 = time.perf_counter()
        st = self.ions.update_fields(cfg.dt, stats=True, sample=sample)
        t2 = time.perf_counter()
        self.solver.update_rho()
        _, sst = self.solver.solve()
        self.solver.update_gradient_field()
        t3 = time.perf_counter()
        self.timings["source"] += t1 - t0
        self.timings["push"] += t2 - t1
        self.timings["solve"] += t3 - t2
        self.solve_stats.append(sst)
        self.it += 1
        return st, sst

    def run(self, steps):
        out = []
        for _ in range(steps):
            out.append(self.step())
        return out

    def close(self):
        self.dom.close()
