"""Benchmark: particle push + charge scatter on the 2049x1025 / 64M-ion ES-PIC workload.

One step = KineticMaterial.updateFields() for the ion species on the GPU: E gather,
velocity update, move, surface/exit handling, deterministic int64 node scatter, density
finalisation, plus the automatic cell sort every 16 steps (amortised inside the timed
steps).  Metric: particle-steps/s (whole job).  The particle arrays (64M x 24 B =
1.6 GB) are far larger than L2 (129 MB), so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference algorithm's CPU restatement (the oracle port; the
Java reference cannot run here) on the host cores with a bounded sample of the same
workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (push+scatter); Poisson ms/solve to 1e-6 residual"
UNIT = "particle-steps/s"
# algorithmic bytes: per particle-step read cell, fx, fy, vx, vy (20 B) + write them (20 B);
# per node per push launch: E read (8 B) + int64 count read-modify-write via atomics (16 B)
BYTES_PER_PARTICLE = 40
BYTES_PER_NODE_PUSH = 24


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def setup_workload(n_particles, seed=0):
    from starfish_gb300 import workloads as W
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    cfg = W.config1(n_particles)
    spec = cfg.mesh
    _, efi, efj = W.electrode_efield(spec)
    dom = GpuDomain(spec, device=0)
    dom.set_efield(efi, efj)
    km = KineticMaterial(dom, cfg.ion.mass, cfg.ion.charge, cfg.ion.spwt,
                         capacity=int(n_particles * 1.1) + 1024)
    chunk = 8 * 1024 * 1024
    for c0 in range(0, n_particles, chunk):
        m = min(chunk, n_particles - c0)
        pos, vel = W.uniform_maxwellian(spec, cfg.ion, m, seed + c0)
        km.add_particles(pos, vel, rewind=True, dt=cfg.dt)
    # no explicit sort: the first push sorts (automatically, with the look-ahead key of
    # the steps that follow), so the timed steps see the steady-state sort cycle
    return cfg, dom, km, efi, efj


def electrode_potential(step, period=2000):
    """Electrode potential of the learned-warm-start workload: -100 - 100 cos(2 pi t / T) V."""
    return -100.0 - 100.0 * np.cos(2 * np.pi * step / period)


def learned_poisson_bench(cfg, dom, km, steps=2000, train_steps=500, compare_every=10, tol=1e-6,
                          base=32, down=8, keep_training_every=0, mode=1):
    """Learned-warm-start workload on the 2049x1025 mesh: the full ES-PIC step (Maxwellian
    inlet at x = 0, push + scatter of the ions, rho, Poisson-Boltzmann solve, E) with the
    electrode potential following -100 - 100 cos(2 pi t / 2000) V.  The U-Net trains online
    on the first `train_steps` solves; from then on every solve starts from its prediction
    and, every `compare_every` steps, the same solve is repeated plain (from the same
    previous potential), so both are timed on identical inputs and reach the same FP64
    residual ||R||_2/N < tol.  Solve times are CUDA-event device times of sf_poisson_nl
    (the learned one includes the network's inference and the residual of the previous
    potential it is checked against).  keep_training_every > 0 keeps training online
    after the training phase on one pair every that many solves (outside the timing).
    mode 2 uses the network as the coarse correction inside the PCG instead of as the
    start: it trains on the first residual of each converged solve (use_learned = 2 from
    the first step, the correction switching on once trained), and the compared solves
    start from the same previous potential with and without the correction."""
    from starfish_gb300 import abi
    from starfish_gb300.plugin import LearnedWarmStart, PoissonSolver
    spec = cfg.mesh
    Lx, Ly = spec.lengths()
    inlet = np.array([spec.x0[0], spec.x0[1] + Ly, spec.x0[0], spec.x0[1]])
    ps = PoissonSolver(dom, n0=cfg.n0, Te0=cfg.Te0, phi0=cfg.phi0, tol=tol, max_it=60, cycles=4)
    net = LearnedWarmStart(dom, base=base, down=down, seed=0, lr=1e-3, iters_per_sample=1)
    electrode = spec.bc_value != 0
    bc = spec.bc_value.copy()
    ion = cfg.ion
    cold = None
    plain, learned, learned_all = [], [], []
    if mode == 2:
        ps.use_learned(True, mode=2)  # trains on every converged solve until train_steps
    t_start = time.perf_counter()
    for t in range(steps):
        bc[electrode] = electrode_potential(t)
        ps.set_bc_values(bc)
        km.sample_maxwellian_source(inlet, ion.den, ion.v_drift, ion.temp, cfg.dt)
        km.update_fields(cfg.dt, stats=False)
        ps.update_rho()
        if t == train_steps:
            if keep_training_every > 0:
                net.train(True, lr=1e-3, every=keep_training_every)
            else:
                net.train(False)
            ps.use_learned(True, mode=mode)
        compare = t >= train_steps and (t - train_steps) % compare_every == 0
        phi_prev = dom.get_field(abi.FIELD_PHI) if compare else None
        _, st = ps.solve()
        if t == 0:
            cold = st
        if t >= train_steps:
            learned_all.append(st)
        if compare:
            learned.append(st)
            ps.use_learned(False)
            _, sp = ps.solve(phi=phi_prev)
            ps.use_learned(True, mode=mode)
            plain.append(sp)
        ps.update_gradient_field()
    wall = time.perf_counter() - t_start
    ns = net.stats()

    def mean(lst, k):
        return float(np.mean([x[k] for x in lst])) if lst else None

    pm, lm = mean(plain, "ms"), mean(learned, "ms")
    return {"metric": "Poisson ms/solve to ||R||_2/N < 1e-6 (FP64), learned vs plain " +
                      ("warm start" if mode == 1 else "preconditioner (no learned coarse correction)"),
            "mode": "warm start" if mode == 1 else "coarse correction inside the PCG",
            "tensor_core_convs": net.tensor_core_convs(),
            "plain_ms": pm, "learned_ms": lm, "speedup": (pm / lm) if pm and lm else None,
            "plain_newton_it": mean(plain, "newton_it"), "learned_newton_it": mean(learned, "newton_it"),
            "plain_initial_residual": mean(plain, "initial_residual"),
            "learned_initial_residual": mean(learned, "initial_residual"),
            "learned_ms_all_steps": mean(learned_all, "ms"), "compared_solves": len(plain),
            "max_residual": max([x["residual"] for x in plain + learned], default=None),
            "cold_start_ms": cold["ms"], "cold_start_newton_it": cold["newton_it"],
            "training": {"solves": ns["samples"], "ms_per_solve": ns["train_ms"] / max(ns["samples"], 1),
                         "final_loss": ns["loss"], "network": f"U-Net 4 levels, base {base}, "
                         f"grid {net.Wn}x{net.Hn} (mesh / {down}), BF16 3x3 convolutions on tcgen05 "
                         f"(mma.sync where the grid row is not 16/32/64/128k), Adam lr 1e-3",
                         "keep_training_every": keep_training_every},
            "predictions_used": ns["used"], "predictions_rejected": ns["rejected"],
            "steps": steps, "train_steps": train_steps, "electrode": "-100 - 100 cos(2 pi t / 2000) V",
            "mesh": [spec.ni, spec.nj], "tol": tol, "particles_end": km.get_np(), "wall_s": wall}


def l2_copy_gbs(mb=24, reps=200):
    """Copy bandwidth of a buffer that stays in L2 (two 24 MB buffers, 129 MB of L2): the
    reference for kernels whose grids are L2-resident (torch copy on the device)."""
    import torch
    n = mb * 1024 * 1024 // 4
    a = torch.ones(n, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    for _ in range(10):
        b.copy_(a)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        b.copy_(a)
    e1.record()
    e1.synchronize()
    return 2 * 4 * n * reps / (e0.elapsed_time(e1) / 1e3) / 1e9


def poisson_roofline(cfg, dom, solves=4, tol=1e-6):
    """Per-kernel roofline of the plain solve on this mesh: the solve's launches run with
    per-kernel CUDA events (outside the CUDA graph the timed solves use; the kernels are
    the same) over `solves` warm solves, each after a 20 V step of the electrode.
    Algorithmic bytes per launch: multigrid level l going down reads r, P (FP32) and the
    node class (1 B) and writes y per fine node, and writes the restricted residual per
    coarse node (13 + 4 N_{l+1}/N_l B per node); going up it reads the coarse correction,
    y, r, P and the class and writes y (17 + 4 N_{l+1}/N_l B); the FP64 Newton residual
    reads phi, b0 (FP64) and the class and writes F and P (FP32): 25 B per node, and runs
    about 20 FP64 instructions per node (FP64-pipe-bound), reported against the part's
    nominal FP64 rate."""
    from starfish_gb300.plugin import PoissonSolver
    ps = PoissonSolver(dom, n0=cfg.n0, Te0=cfg.Te0, phi0=cfg.phi0, tol=tol, max_it=60, cycles=4)
    ni, nj = cfg.mesh.ni, cfg.mesh.nj
    levels = [(ni, nj)]
    while levels[-1][0] * levels[-1][1] > 2200 and (levels[-1][0] - 1) % 2 == 0 and (levels[-1][1] - 1) % 2 == 0:
        a, b = levels[-1]
        levels.append(((a - 1) // 2 + 1, (b - 1) // 2 + 1))
    bc = cfg.mesh.bc_value.copy()
    electrode = bc != 0
    ps.set_bc_values(bc)
    ps.solve()  # settle
    dom.timing(True)
    dom.timing_reset()
    for k in range(solves):
        # warm solves that have work to do: the electrode moves by 20 V between them
        bc[electrode] = -100.0 - 20.0 * ((k % 2) + 1)
        ps.set_bc_values(bc)
        ps.solve()
    peak, kind = measured_peaks()
    l2 = l2_copy_gbs()
    out = {"kernels": {}, "hbm_peak_gbs": peak, "peak_kind": kind, "l2_copy_gbs": l2,
           "how": "per-kernel CUDA events over warm plain solves on the 2049x1025 mesh"}
    for l in range(len(levels) - 1):
        nf = levels[l][0] * levels[l][1]
        nc = levels[l + 1][0] * levels[l + 1][1]
        for name, per_node in ((f"mg_down_L{l}", 13), (f"mg_up_L{l}", 17)):
            ms, cnt = dom.kernel_time(name)
            if cnt == 0:
                continue
            b = per_node * nf + 4 * nc
            gbs = b / (ms / cnt / 1e3) / 1e9
            out["kernels"][name] = {"nodes": nf, "ms": ms / cnt, "launches": cnt, "alg_bytes": b, "gbs": gbs,
                                    "frac_hbm": gbs / peak, "frac_l2": gbs / l2}
    ms, cnt = dom.kernel_time("nl_residual")
    if cnt:
        b = 25 * ni * nj
        gbs = b / (ms / cnt / 1e3) / 1e9
        # FP64 arithmetic instructions per interior node, counted from the kernel's source
        # (5-point operator 6, argument 2, table exponential and its range test 5, coefficient
        # and P 2, F 2, the norm and max 2, the mode test 1); about 7 FP32/FP64 conversions
        # per node come on top.  Against the nominal 1.25 TFLOP/s FP64 of the part (no
        # measured FP64 peak): 0.625e12 FP64 lane-instructions per second.
        fp64_per_node = 20
        ginst = fp64_per_node * ni * nj / (ms / cnt / 1e3) / 1e9
        out["kernels"]["nl_residual"] = {"nodes": ni * nj, "ms": ms / cnt, "launches": cnt, "alg_bytes": b,
                                         "gbs": gbs, "frac_hbm": gbs / peak, "frac_l2": gbs / l2,
                                         "bound": "FP64 pipe",
                                         "fp64_instr_per_node": fp64_per_node, "fp64_ginstr_s": ginst,
                                         "frac_fp64_nominal": ginst / 625.0,
                                         "fp64_peak": "nominal 1.25 TFLOP/s = 625 G FP64 lane-instructions/s"}
    for name in ("mg_coarse", "cg_matvec"):
        ms, cnt = dom.kernel_time(name)
        if cnt:
            out["kernels"][name] = {"ms": ms / cnt, "launches": cnt}
    dom.timing(False)
    return out


def dsmc_jet_bench(steps=20, warmup=3, n_particles=16 * 1024 * 1024, seed=0):
    """The DSMC expanding-jet workload: Argon on the 513x257 axisymmetric (ZR) mesh, inlet
    r < 5 mm at 1e22 m^-3 / 300 K / 500 m/s sampled on the device every step, diffuse
    walls at 300 K, VHS NTC collisions (Bird 4.63 cross-section) per cell, 16M preloaded
    macroparticles.  One step = inlet source + push (with wall hits) + DSMC (counting
    sort into cells + NTC).  Throughput in particle-steps/s over device-resident
    particles; k_dsmc's roofline from 28 B per particle (velocity read + write, cell) plus
    16 B per cell of per-cell state."""
    import torch
    from starfish_gb300 import abi
    from starfish_gb300 import workloads as W
    from starfish_gb300.plugin import DSMC, GpuDomain, KineticMaterial
    cfg = W.config2(n_particles)
    spec = cfg.mesh
    dom = GpuDomain(spec, device=0)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, cfg.mass, 0.0, cfg.spwt, capacity=int(n_particles * 1.3) + 4096)
        vth = np.sqrt(2 * W.KB * cfg.wall_temp / cfg.mass)
        for sidx in range(spec.seg_xy.shape[0]):
            km.set_surface(sidx, abi.SURF_DIFFUSE, vth=vth, c_rest=1.0, c_accom=1.0)
        chunk = 4 * 1024 * 1024
        for c0 in range(0, n_particles, chunk):
            pos, vel = W.jet_particles(cfg, min(chunk, n_particles - c0), seed + c0)
            km.add_particles(pos, vel, rewind=False, dt=cfg.dt)
        ds = DSMC(dom, km, model=abi.SIGMA_BIRD463, diam=cfg.diam, T_ref=cfg.T_ref, omega=cfg.omega)

        def step():
            # the source, the push and the collisions are queued without a host read; the
            # cell sort still reads its particle count back
            km.sample_maxwellian_source(cfg.inlet, cfg.den, cfg.v_drift, cfg.temp, cfg.dt, wait=False)
            km.update_fields(cfg.dt, stats=False, wait=False)
            ds.perform(cfg.dt, wait=False)

        for _ in range(max(warmup, 3)):
            step()
        ext = torch.cuda.ExternalStream(dom.stream())
        dom.timing(True)
        dom.timing_reset()
        l0 = dom.launches()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ps0 = km.particle_steps()
        c0 = ds.counts()[0].sum()
        e0.record(ext)
        for _ in range(steps):
            step()
        e1.record(ext)
        e1.synchronize()
        psteps = km.particle_steps() - ps0
        colls = ds.counts()[0].sum() - c0
        ms = e0.elapsed_time(e1)
        launches = dom.launches() - l0
        k = {name: dom.kernel_time(name) for name in ("push", "push_slow", "sort", "finalize", "dsmc")}
        dom.timing(False)
        avg_np = psteps / steps
        nc_cells = (spec.ni - 1) * (spec.nj - 1)
        dsmc_ms = k["dsmc"][0] / max(k["dsmc"][1], 1)
        alg = 28.0 * avg_np + 16.0 * nc_cells
        peak, peak_kind = measured_peaks()
        return {"metric": "particle-steps/s (source + push + DSMC)", "value": psteps / (ms / 1e3),
                "unit": "particle-steps/s", "ms_per_step": ms / steps, "steps": steps,
                "workload": cfg.name, "mesh": [spec.ni, spec.nj], "particles_avg": avg_np,
                "collisions_per_step": colls / steps, "dt_s": cfg.dt,
                "kernel_ms": {n: v[0] / max(v[1], 1) for n, v in k.items()},
                "roofline_dsmc": {"bound": "hbm", "achieved": alg / (dsmc_ms / 1e3) / 1e9, "peak": peak,
                                  "unit": "GB/s", "frac": alg / (dsmc_ms / 1e3) / 1e9 / peak,
                                  "peak_kind": peak_kind, "alg_bytes_per_launch": alg},
                "gpu_launches": launches}
    finally:
        dom.close()


def batch_bench(n_instances=256, steps=16, warmup=10, threads=16, dt=5e-7, unbatched_steps=3):
    """The batched-instances workload: 256 independent 81x41-type ES-PIC cases (mesh sizes
    log-uniform from 33x17 to 257x129 nodes, 1e4..2e6 preloaded ions each, electrode at
    -200..-20 V, O+ inlet, seeds 0..255) advanced together by sf_batch_step: batched
    sources + one push launch over all instances (replayed as one CUDA graph), then every
    instance's rho, Poisson-Boltzmann solve to 1e-6 and E, overlapping from `threads` host
    threads.  The warm-up steps include the autotuner's trials.  Throughput: live
    particles of all instances x steps / wall time of the steps."""
    from starfish_gb300 import workloads as W
    from starfish_gb300.plugin import GpuBatch, GpuDomain, KineticMaterial, PoissonSolver
    cases = W.config4(n_instances)
    doms, kms, solvers = [], [], []
    t_setup = time.perf_counter()
    for c in cases:
        spec, ion = c.mesh, c.ion
        dom = GpuDomain(spec, device=0)
        ps = PoissonSolver(dom, n0=1e12, Te0=2.0, tol=1e-6, max_it=60)
        ps.solve(rho=np.zeros(spec.nn), phi=np.zeros(spec.nn))
        ps.update_gradient_field()
        Lx, Ly = spec.lengths()
        v_mean = np.sqrt(8 * W.KB * ion.temp / (np.pi * ion.mass))
        inject = 1e12 * Ly * (ion.v_drift + v_mean / 4) * dt / ion.spwt
        # removed slots stay until the sort every 16 steps
        km = KineticMaterial(dom, ion.mass, ion.charge, ion.spwt,
                             capacity=int(1.3 * c.n_particles + 24 * inject) + 8192)
        pos, vel = W.uniform_maxwellian(spec, ion, c.n_particles, c.seed)
        km.add_particles(pos, vel, rewind=True, dt=dt)
        doms.append(dom)
        kms.append(km)
        solvers.append(ps)
    batch = GpuBatch(doms, kms, threads=threads)
    try:
        for i, c in enumerate(cases):
            Lx, Ly = c.mesh.lengths()
            batch.set_source(i, [0.0, Ly, 0.0, 0.0], c.ion.den, c.ion.v_drift, c.ion.temp)
        t_setup = time.perf_counter() - t_setup
        for _ in range(warmup):
            batch.step(dt, solvers[0])
        psteps, dev_ms, solve_sum, solve_max, newton, newton_max = 0, 0.0, 0.0, 0.0, 0.0, 0
        live = sum(km.get_np() for km in kms)
        t0 = time.perf_counter()
        for _ in range(steps):
            psteps += live
            st = batch.step(dt, solvers[0])
            live = st["particles"]
            dev_ms += st["device_phase_ms"]
            solve_sum += st["solve_ms_sum"]
            solve_max = max(solve_max, st["solve_ms_max"])
            newton += st["newton_it_mean"]
            newton_max = max(newton_max, st["newton_it_max"])
        wall = time.perf_counter() - t0
        tuning = batch.tuning()
        batch.close()
        # the same instances afterwards, one at a time through the per-instance entry
        # points (source, push + scatter, rho, Poisson with the tuned PCG iterations, E)
        ps_u, wall_u = 0, 0.0
        if unbatched_steps > 0:
            for c, ps in zip(cases, solvers):
                nn = c.mesh.nn
                ps.prm.cycles = tuning["pcg_iterations_by_bucket"][0 if nn < 4096 else (1 if nn < 16384 else 2)]
            live_u = sum(km.get_np() for km in kms)
            t1 = time.perf_counter()
            for _ in range(unbatched_steps):
                ps_u += live_u
                live_u = 0
                for c, km, ps in zip(cases, kms, solvers):
                    Ly = c.mesh.lengths()[1]
                    km.sample_maxwellian_source(np.array([0.0, Ly, 0.0, 0.0]), c.ion.den, c.ion.v_drift,
                                                c.ion.temp, dt)
                    km.update_fields(dt, stats=False)
                    ps.update_rho()
                    ps.solve()
                    ps.update_gradient_field()
                    live_u += km.get_np()
            wall_u = time.perf_counter() - t1
        sizes = [c.mesh.nn for c in cases]
        return {"metric": "particle-steps/s over all instances (source + push + scatter + Poisson + E)",
                "value": psteps / wall, "unit": "particle-steps/s", "ms_per_step": 1e3 * wall / steps,
                "steps": steps, "warmup": warmup, "instances": n_instances,
                "particles_live_end": live, "mesh_nodes": [min(sizes), max(sizes)],
                "device_phase_ms": dev_ms / steps, "solve_ms_sum_per_step": solve_sum / steps,
                "solve_ms_max": solve_max, "newton_it_mean": newton / steps, "newton_it_max": newton_max,
                "host_threads": threads, "tuning": tuning, "setup_s": t_setup,
                "timing": "wall clock of sf_batch_step (host threads and graph launches included)",
                "unbatched": None if unbatched_steps <= 0 else {
                    "value": ps_u / wall_u, "ms_per_step": 1e3 * wall_u / unbatched_steps,
                    "steps": unbatched_steps,
                    "how": "the same contexts after the batched steps, each instance stepped in turn "
                           "from one host thread through the per-instance entry points"}}
    finally:
        batch.close()
        for d in doms:
            d.close()


def cpu_baseline_sample(cfg, efi, efj, n_sample, threads, steps=1, seed=1):
    """The oracle port (reference algorithm, FP64 AoS) on a bounded sample of the workload."""
    from oracle import oracle as O
    from starfish_gb300 import workloads as W
    spec = cfg.mesh
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    pos, vel = W.uniform_maxwellian(spec, cfg.ion, n_sample, seed)
    P = np.zeros((n_sample, 12))
    P[:, 0:2] = pos[:, 0:2]
    P[:, 3:6] = vel
    P[:, 6] = (pos[:, 0] - spec.x0[0]) / spec.dh[0]
    P[:, 7] = (pos[:, 1] - spec.x0[1]) / spec.dh[1]
    P[:, 9] = cfg.ion.spwt
    P[:, 10] = 1
    vol = O.node_volumes(m)
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_ABSORB)
    if spec.node_seg_ptr is None:
        spec.node_seg_ptr, spec.node_seg_idx = O.node_segments(m, spec.seg_xy)
    done = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        n_alive = int((P[:, 10] == 1).sum())
        O.push(m, efi, efj, cfg.ion.charge, cfg.ion.mass, cfg.dt, segs, spec.node_seg_ptr,
               spec.node_seg_idx, P, threads=threads)
        O.update_fields(m, vol, P)
        done += n_alive
    t = time.perf_counter() - t0
    return done / t, t


def aggregate_over_ranks(ms, psteps, device):
    """One replica per rank: the slowest rank's timed milliseconds and the particle-steps of
    all ranks, over the default process group."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    tot = torch.tensor([float(psteps)], dtype=torch.float64, device=device)
    dist.all_reduce(tot)
    return t.item(), tot.item()


POISSON_PAIR_MESH = (257, 129)


def poisson_pair_inputs(seed=3):
    """The field-solve case timed on both arms: the ES-PIC geometry (phi = 0 walls, the
    centred -100 V electrode) on a 257x129 mesh over the same 80 mm x 40 mm, with a noisy
    ion charge density around e * 1e12 m^-3, solved from phi = 0."""
    from starfish_gb300 import workloads as W
    ni, nj = POISSON_PAIR_MESH
    spec = W.es_pic_mesh(ni, nj, 80e-3 / (ni - 1))
    rng = np.random.default_rng(seed)
    rho = 1.602176565e-19 * 1e12 * (1 + 0.2 * rng.standard_normal(spec.nn))
    return spec, rho


def reference_poisson_solve(seed=3):
    """The oracle's Newton + SOR (omega 1.4; PoissonSolver / LinearSolverGS defaults: Newton
    tolerance 1e-4, linear tolerance 1e-6 on ||R||_2/N) on poisson_pair_inputs, one host
    core (the reference's solver sweeps its rows in one thread per mesh)."""
    from oracle import oracle as O
    spec, rho = poisson_pair_inputs(seed)
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    t0 = time.perf_counter()
    phi, it, out = O.poisson_nl(m, spec.bc_value, rho, 1e12, 2.0, 0.0, 8.85418782e-12, np.zeros(spec.nn),
                                max_it=2000000, tol=1e-6, nl_max_it=100, nl_tol=1e-4)
    ms = 1e3 * (time.perf_counter() - t0)
    res = O.poisson_residual(m, spec.bc_value, rho, 1e12, 2.0, 0.0, 8.85418782e-12, phi) / spec.nn
    return {"workload": f"es_pic_{spec.ni}x{spec.nj} solve from phi = 0", "ms_per_solve": ms,
            "newton_it": int(it), "linear_sweeps": int(out[1]), "residual": float(res), "cores": 1,
            "kind": "port"}


def gpu_poisson_solve(seed=3, repeats=5):
    """sf_poisson_nl on poisson_pair_inputs from phi = 0 to ||R||_2/N < 1e-6 (FP64): one
    untimed solve (graph capture), then the median CUDA-event time of `repeats` solves."""
    from starfish_gb300.plugin import GpuDomain, PoissonSolver
    spec, rho = poisson_pair_inputs(seed)
    dom = GpuDomain(spec, device=0)
    try:
        ps = PoissonSolver(dom, n0=1e12, Te0=2.0, phi0=0.0, tol=1e-6, max_it=60, cycles=4)
        zero = np.zeros(spec.nn)
        ps.solve(rho=rho, phi=zero)
        sts = [ps.solve(rho=rho, phi=zero)[1] for _ in range(repeats)]
    finally:
        dom.close()
    ms = sorted(x["ms"] for x in sts)[len(sts) // 2]
    return {"workload": f"es_pic_{spec.ni}x{spec.nj} solve from phi = 0", "ms_per_solve": ms,
            "newton_it": sts[0]["newton_it"], "residual": max(x["residual"] for x in sts), "repeats": repeats}


def reference_dsmc_jet(n_particles=16 * 1024 * 1024, steps=1, warmup=2, threads=None, seed=0):
    """The oracle's jet step on the DSMC leg's workload (513x257 ZR, 16M argon preloaded like
    the GPU leg; fewer macroparticles scale the weight up, which keeps the candidates per
    particle, nsel ~ n^2 w / V per cell, and so the work per particle-step, about the
    same).  Each step: the inlet source, the push with
    diffuse walls on `threads` host threads, then DSMC.perform (one host thread: the
    reference's collideCell loop is serial).  `warmup` untimed steps first let (sigma g)max
    grow from its initial 1e-16, as the GPU leg's warm-up steps do.  Particle-steps/s over
    the timed steps, and the DSMC call's own time."""
    from oracle import oracle as O
    from starfish_gb300 import workloads as W
    cfg = W.config2(n_particles)
    spec = cfg.mesh
    threads = threads or os.cpu_count() or 1
    m = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
    ptr, idx = O.node_segments(m, spec.seg_xy)
    cv = O.cell_volumes(m)
    vth = np.sqrt(2 * W.KB * cfg.wall_temp / cfg.mass)
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_DIFFUSE, vth=vth, c_rest=1.0, c_accom=1.0)
    zero = np.zeros(spec.nn)
    pos, vel = W.jet_particles(cfg, n_particles, seed)
    P = np.zeros((n_particles, 12))
    P[:, 0:3] = pos
    P[:, 3:6] = vel
    P[:, 9] = cfg.spwt
    O.add_particles(m, zero, zero, 0.0, cfg.mass, cfg.dt, P)
    nc = (spec.ni - 1) * (spec.nj - 1)
    state = np.zeros((nc, 2))
    state[:, 0] = 1e-16
    counts = np.zeros((nc, 2))
    rem, done, t_all, t_dsmc, c0 = 0.0, 0, 0.0, 0.0, 0.0
    for t in range(warmup + steps):
        if t == warmup:
            done, t_all, t_dsmc, c0 = 0, 0.0, 0.0, float(counts[:, 0].sum())
        t0 = time.perf_counter()
        new, rem = O.maxwellian_source(seed * 1000003 + t, cfg.inlet, cfg.den, cfg.v_drift, cfg.temp, cfg.mass,
                                       cfg.spwt, cfg.dt, rem, domain=spec.domain)
        O.add_particles(m, zero, zero, 0.0, cfg.mass, cfg.dt, new)
        P = np.ascontiguousarray(np.vstack([P, new]))
        done += P.shape[0]
        O.push(m, zero, zero, 0.0, cfg.mass, cfg.dt, segs, ptr, idx, P, seed=seed * 7919 + t, threads=threads)
        P = np.ascontiguousarray(P[P[:, 10] == 1])
        t1 = time.perf_counter()
        O.dsmc(spec.ni, spec.nj, cv, P, cfg.mass, cfg.spwt, cfg.diam, cfg.T_ref, cfg.omega, 1.0, cfg.dt,
               state, counts, seed * 104729 + t)
        t2 = time.perf_counter()
        t_all += t2 - t0
        t_dsmc += t2 - t1
    return {"workload": cfg.name, "value": done / t_all, "unit": "particle-steps/s (source + push + DSMC)",
            "ms_per_step": 1e3 * t_all / steps, "dsmc_ms_per_step": 1e3 * t_dsmc / steps,
            "collisions_per_step": float((counts[:, 0].sum() - c0) / steps), "steps": steps, "warmup": warmup,
            "sample": f"{n_particles} macroparticles, {warmup} untimed + {steps} timed steps",
            "cores": {"push": threads, "dsmc": 1}, "kind": "port"}


def workload_config(cfg, particles, world):
    """The `config` of both arms' lines: the workload they measure."""
    return {"workload": cfg.name, "mesh": [cfg.mesh.ni, cfg.mesh.nj], "dx_m": cfg.mesh.dh[0],
            "particles_per_gpu": particles, "dt_s": cfg.dt, "sort_interval": 16,
            "l2": "inputs larger than L2 (1.6 GB of particles per step)", "parallelism": f"replicas x{world}"}


def run_reference(args):
    """Reference arm: the CPU restatement with all host threads, on the same workload and
    metric.  Each timed step pushes and scatters a bounded sample of the 64M ions (the
    whole population would take minutes per step on the host); `ms_per_step` is the
    time of those sampled steps as measured, and the rate is sampled particle-steps over
    that time.  The field solve is timed on the 257x129 case that the GPU arm also solves."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from starfish_gb300 import workloads as W
    n_particles = 64 * 1024 * 1024
    cfg = W.config1(n_particles)
    _, efi, efj = W.electrode_efield(cfg.mesh)
    threads = os.cpu_count() or 1
    n_sample = 4 * 1024 * 1024
    for _ in range(max(args.warmup, 0) and 1):
        cpu_baseline_sample(cfg, efi, efj, n_sample // 8, threads, 1)
    vals = []
    for k in range(args.steps):
        v, t = cpu_baseline_sample(cfg, efi, efj, n_sample, threads, 1, seed=k + 1)
        vals.append((v, t))
    total_ps = n_sample * args.steps
    total_t = sum(t for _, t in vals)
    value = total_ps / total_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(cfg, n_particles, args.gpus),
        "timed_sample": {"particles_per_step": n_sample, "of_particles": n_particles,
                         "note": "ms_per_step is the measured time of a step over the sample"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_sample} of the {n_particles} ions per step, "
                                   f"{args.steps} steps, push on {threads} threads + serial scatter"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "poisson": reference_poisson_solve(),
        "dsmc": reference_dsmc_jet(),
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--particles", type=int, default=64 * 1024 * 1024)
    ap.add_argument("--burn-in", type=int, default=0,
                    help="untimed pushes after set-up, before the warm-up (the population decays "
                         "as ions leave the domain: 64M at set-up, about 50M after 35 steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--poisson-steps", type=int, default=2000)
    ap.add_argument("--dsmc-steps", type=int, default=20)
    ap.add_argument("--precond-steps", type=int, default=1000,
                    help="steps of the learned coarse-correction leg (0: skip)")
    ap.add_argument("--no-poisson-pair", dest="poisson_pair", action="store_false",
                    help="skip the 257x129 solve that the reference arm also times")
    ap.add_argument("--batch-steps", type=int, default=16)
    ap.add_argument("--batch-threads", type=int, default=16)
    ap.add_argument("--batch-instances", type=int, default=256)
    ap.add_argument("--batch-warmup", type=int, default=10)
    ap.add_argument("--batch-unbatched-steps", type=int, default=3)
    ap.add_argument("--only-batch", action="store_true",
                    help="run only the batched-instances leg and print its result line")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.only_batch:
        from starfish_gb300 import build as B
        B.build()
        print(json.dumps(batch_bench(n_instances=args.batch_instances, steps=args.batch_steps,
                                     warmup=args.batch_warmup, threads=args.batch_threads,
                                     unbatched_steps=args.batch_unbatched_steps)))
        return

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from starfish_gb300 import build as B
    B.build()

    cfg, dom, km, efi, efj = setup_workload(args.particles, seed=1000 * rank)
    ext = torch.cuda.ExternalStream(dom.stream())
    W_ = max(args.warmup, 3) if args.warmup >= 0 else 3
    # optional burn-in; the first push sorts the preloaded ions (random order) with the
    # look-ahead key, so the warm-up and timed pushes already follow the sort cycle
    for _ in range(max(args.burn_in, 0) + W_):
        km.update_fields(cfg.dt, stats=False)

    # ---- timed region: device-resident particles (value) ----
    dom.timing(True)
    dom.timing_reset()
    launches0 = dom.launches()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    # the pushes are queued without waiting (SF_PUSH_NOWAIT), as a time loop that hands
    # the density to the field solve on the same stream would; the species' particle-step
    # counter gives the particles alive at the start of every timed push
    ps0 = km.particle_steps()
    ev0.record(ext)
    for _ in range(args.steps):
        km.update_fields(cfg.dt, stats=False, wait=False)
    ev1.record(ext)
    ev1.synchronize()
    torch.cuda.synchronize()
    psteps = km.particle_steps() - ps0
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    launches = dom.launches() - launches0
    push_ms, push_n = dom.kernel_time("push")
    fin_ms, fin_n = dom.kernel_time("finalize")
    sort_ms, sort_n = dom.kernel_time("sort")
    slow_ms, slow_n = dom.kernel_time("push_slow")
    dom.timing(False)
    if world > 1:
        ms, psteps_all = aggregate_over_ranks(ms, psteps, "cuda")
    else:
        psteps_all = float(psteps)
    value = psteps_all / (ms / 1e3)

    # ---- end-to-end through the C ABI with host buffers ----
    efi_h = torch.from_numpy(efi.copy()).pin_memory().numpy()
    efj_h = torch.from_numpy(efj.copy()).pin_memory().numpy()
    nd_h = torch.zeros(cfg.mesh.nn, dtype=torch.float64).pin_memory().numpy()
    from starfish_gb300 import abi
    lib = dom.lib
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # per step: E in from pinned host buffers, the push queued, the density read back
    # (which waits for the push); particle-steps from the species' counter
    ps0 = km.particle_steps()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dom.check(lib.sf_set_efield(dom.ctx, abi.ptr(efi_h), abi.ptr(efj_h)))
        dom.check(lib.sf_push_deposit(dom.ctx, km.sid, cfg.dt, abi.PUSH_NOWAIT, None))
        dom.check(lib.sf_get_field(dom.ctx, abi.FIELD_ND, km.sid, abi.ptr(nd_h)))
    e2e_s = time.perf_counter() - t0
    e_steps = km.particle_steps() - ps0
    e2e_val = e_steps * world / e2e_s

    peak, peak_kind = measured_peaks()
    nn = cfg.mesh.nn
    avg_np = psteps / max(args.steps, 1)
    push_avg_ms = push_ms / max(push_n, 1)
    alg_bytes = BYTES_PER_PARTICLE * avg_np + BYTES_PER_NODE_PUSH * nn
    achieved = alg_bytes / (push_avg_ms / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "push_traffic.json")
    if os.path.exists(tf):
        try:
            tr = json.load(open(tf))
            traffic = tr["bytes_per_particle"] * avg_np + tr.get("bytes_per_node", 0) * nn
        except Exception:
            traffic = None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": W_, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(cfg, args.particles, world),
        "burn_in_steps": max(args.burn_in, 0),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "k_push", "alg_bytes_per_launch": alg_bytes,
                     "avg_launch_ms": push_avg_ms},
        "kernel_ms": {"push": push_ms / max(push_n, 1), "push_slow": slow_ms / max(slow_n, 1),
                      "finalize": fin_ms / max(fin_n, 1), "sort": sort_ms / max(sort_n, 1),
                      "sort_launches": sort_n},
        "clocks": clk,
        "gpu_launches": launches,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * nn,
                "d2h_bytes_per_step": 8 * nn + 64},
    }
    # ---- field solve on the same mesh: the learned-warm-start workload (full ES-PIC steps
    # with a sinusoidal electrode), learned vs plain solves on identical inputs ----
    if args.poisson_steps > 0:
        line["poisson"] = learned_poisson_bench(cfg, dom, km, steps=args.poisson_steps,
                                                train_steps=min(500, args.poisson_steps // 4))
        if args.precond_steps > 0:
            line["poisson_precond"] = learned_poisson_bench(cfg, dom, km, steps=args.precond_steps,
                                                            train_steps=min(300, args.precond_steps // 3),
                                                            mode=2)
        line["roofline_poisson"] = poisson_roofline(cfg, dom)
    if args.poisson_pair:
        # the same solve as the reference arm's `poisson` (257x129 from phi = 0)
        line["poisson_257x129"] = gpu_poisson_solve()
    if args.dsmc_steps > 0:
        line["dsmc"] = dsmc_jet_bench(steps=args.dsmc_steps)
    if args.batch_steps > 0:
        line["batch"] = batch_bench(n_instances=args.batch_instances, steps=args.batch_steps, threads=args.batch_threads,
                                    unbatched_steps=args.batch_unbatched_steps)
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n_sample = 16 * 1024 * 1024
        v, t = cpu_baseline_sample(cfg, efi, efj, n_sample, threads, steps=2)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{n_sample} particles of the 64M workload, 2 steps "
                                          f"(push on {threads} threads, serial scatter), {t:.1f} s"}
        if args.poisson_pair:
            line["cpu_baseline"]["poisson_257x129"] = reference_poisson_solve()
        if args.dsmc_steps > 0:
            line["cpu_baseline"]["dsmc_jet"] = reference_dsmc_jet()
    dom.close()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
