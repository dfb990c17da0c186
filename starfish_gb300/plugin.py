"""Host-side classes that mirror the reference's plugin surface on top of the C ABI.

``GpuDomain`` stands for the DomainModule/Mesh a Starfish run holds,
``KineticMaterial`` for core/materials/KineticMaterial.java (method names and
argument meaning follow the reference: addParticle, updateFields, getDen ...),
``PoissonSolver`` for pic/PoissonSolver.java, ``DSMC``/``MCC`` for
collisions/DSMC.java and MCC.java.  Every method is one or a few C-ABI calls; no
computation happens here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .workloads import MeshSpec


class GpuDomain:
    def __init__(self, spec: MeshSpec, device: int = 0):
        self.lib = abi.load()
        self.spec = spec
        self._desc = spec.desc()
        h = C.c_void_p()
        rc = self.lib.sf_ctx_create(C.byref(self._desc), device, C.byref(h))
        abi.check(rc, None)
        self.ctx = h
        self.ni, self.nj = spec.ni, spec.nj

    def check(self, rc):
        abi.check(rc, self.ctx)

    def set_seed(self, seed):
        """Starfish.random's seed for every random stream of this domain."""
        self.check(self.lib.sf_ctx_set_seed(self.ctx, int(seed)))

    def set_efield(self, efi, efj):
        efi = np.ascontiguousarray(efi, np.float64)
        efj = np.ascontiguousarray(efj, np.float64)
        self.check(self.lib.sf_set_efield(self.ctx, abi.ptr(efi), abi.ptr(efj)))

    def get_field(self, field, sid=0):
        out = np.zeros(self.ni * self.nj)
        self.check(self.lib.sf_get_field(self.ctx, field, sid, abi.ptr(out)))
        return out

    def stream(self):
        s = C.c_void_p()
        self.check(self.lib.sf_ctx_get_stream(self.ctx, C.byref(s)))
        return s.value

    def timing(self, on=True):
        self.check(self.lib.sf_timing_enable(self.ctx, int(on)))

    def timing_reset(self):
        self.check(self.lib.sf_timing_reset(self.ctx))

    def kernel_time(self, name):
        ms = C.c_double()
        n = C.c_int64()
        self.check(self.lib.sf_timing_get(self.ctx, name.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def launches(self, reset=False):
        n = C.c_int64()
        self.check(self.lib.sf_launch_count(self.ctx, C.byref(n), int(reset)))
        return n.value

    def close(self):
        if self.ctx:
            self.lib.sf_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class KineticMaterial:
    """GPU-resident kinetic species (KineticMaterial, core/materials/KineticMaterial.java)."""

    def __init__(self, domain: GpuDomain, mass, charge, spwt, capacity, nd_back=0.0):
        self.d = domain
        sid = C.c_int32()
        domain.check(domain.lib.sf_species_add(domain.ctx, charge, mass, spwt, int(capacity),
                                               nd_back, C.byref(sid)))
        self.sid = sid.value
        self.mass, self.charge, self.spwt = mass, charge, spwt
        self._src_rem = {}

    # KineticMaterial.addParticle(pos, vel) with the -dt/2 velocity rewind
    def add_particles(self, pos, vel, rewind=True, dt=0.0, mpw=None):
        pos = np.ascontiguousarray(pos, np.float64)
        vel = np.ascontiguousarray(vel, np.float64)
        w = None if mpw is None else np.ascontiguousarray(mpw, np.float64)
        n = pos.shape[0]
        self.d.check(self.d.lib.sf_particles_append(self.d.ctx, self.sid, n, abi.ptr(pos),
                                                    abi.ptr(vel), abi.ptr(w), int(rewind), float(dt)))

    def add_particles_lc(self, lc, vel, mpw=None):
        lc = np.ascontiguousarray(lc, np.float64)
        vel = np.ascontiguousarray(vel, np.float64)
        if mpw is not None:
            w = np.ascontiguousarray(mpw, np.float64)
            self.d.check(self.d.lib.sf_particles_append_lc_w(self.d.ctx, self.sid, lc.shape[0], abi.ptr(lc),
                                                             abi.ptr(vel), abi.ptr(w)))
            return
        self.d.check(self.d.lib.sf_particles_append_lc(self.d.ctx, self.sid, lc.shape[0],
                                                       abi.ptr(lc), abi.ptr(vel)))

    def set_weighted(self, on=True):
        """Per-particle weights (Particle.mpw) for this species, before its first particle."""
        self.d.check(self.d.lib.sf_species_set_weighted(self.d.ctx, self.sid, int(bool(on))))

    def sample_maxwellian_source(self, seg_xy, den, v_drift, temp, dt, wait=True):
        """MaxwellianSource on one straight segment, sampled on the device; returns the
        number of particles added (the fractional remainder is kept per source).  wait=False
        queues the draws and returns None."""
        key = tuple(np.asarray(seg_xy, np.float64).reshape(-1))
        rem = C.c_double(self._src_rem.get(key, 0.0))
        seg = np.ascontiguousarray(seg_xy, np.float64).reshape(-1)
        n = C.c_int64()
        self.d.check(self.d.lib.sf_source_maxwellian(self.d.ctx, self.sid, abi.ptr(seg), den, v_drift,
                                                     temp, dt, C.byref(rem), C.byref(n) if wait else None))
        self._src_rem[key] = rem.value
        return n.value if wait else None

    def sample_uniform_source(self, seg_xy, mdot, v_drift, dt):
        """UniformSource on one straight segment: mass flow rate mdot (kg/s), cold beam
        along the segment normal; returns the number of particles added."""
        key = ("uniform",) + tuple(np.asarray(seg_xy, np.float64).reshape(-1))
        rem = C.c_double(self._src_rem.get(key, 0.0))
        seg = np.ascontiguousarray(seg_xy, np.float64).reshape(-1)
        n = C.c_int64()
        self.d.check(self.d.lib.sf_source_uniform(self.d.ctx, self.sid, abi.ptr(seg), float(mdot), float(v_drift),
                                                  float(dt), C.byref(rem), C.byref(n)))
        self._src_rem[key] = rem.value
        return n.value

    def preload(self, den, temp, dt):
        """VolumePreloadSource: fills every cell at density den (m^-3), temperature temp (K);
        returns the number of particles added."""
        n = C.c_int64()
        self.d.check(self.d.lib.sf_source_preload(self.d.ctx, self.sid, float(den), float(temp), float(dt),
                                                  C.byref(n)))
        return n.value

    def set_surface(self, seg, model, vth=0.0, c_rest=1.0, c_accom=1.0):
        self.d.check(self.d.lib.sf_species_set_surface(self.d.ctx, self.sid, seg, model, vth,
                                                       c_rest, c_accom))

    def set_surface_product(self, seg, product: "KineticMaterial", vth_product=0.0):
        """Species change at segment seg (SPECULAR or DIFFUSE impacts emit the product
        species); product None clears it."""
        self.d.check(self.d.lib.sf_species_set_surface_product(self.d.ctx, self.sid, seg,
                                                               -1 if product is None else product.sid,
                                                               float(vth_product)))

    def set_sort_interval(self, k):
        self.d.check(self.d.lib.sf_species_set_sort_interval(self.d.ctx, self.sid, int(k)))

    def set_sort_block(self, cells):
        """Key of the automatic sort: blocks of cells x cells cells (1, 2, 4, 8, 16)."""
        self.d.check(self.d.lib.sf_species_set_sort_block(self.d.ctx, self.sid, int(cells)))

    def sort(self):
        self.d.check(self.d.lib.sf_particles_sort(self.d.ctx, self.sid))

    def clear(self):
        self.d.check(self.d.lib.sf_particles_clear(self.d.ctx, self.sid))

    # KineticMaterial.updateFields(): push + scatter (+ updateSamples with sample=True)
    def update_fields(self, dt, stats=True, moments=False, sample=False, wait=True):
        """One push + scatter.  wait=False queues it and returns at once (SF_PUSH_NOWAIT;
        without totals the returned counts are -1)."""
        st = abi.PushStats()
        flags = ((abi.PUSH_STATS if stats else 0) | (abi.PUSH_MOMENTS if moments else 0) |
                 (abi.PUSH_SAMPLE if sample else 0) | (0 if wait else abi.PUSH_NOWAIT))
        self.d.check(self.d.lib.sf_push_deposit(self.d.ctx, self.sid, float(dt), flags,
                                                C.byref(st)))
        return st.as_dict()

    def clear_samples(self):
        """KineticMaterial.clearSamples (sets up the sampling buffers on first use)."""
        self.d.check(self.d.lib.sf_samples_clear(self.d.ctx, self.sid))

    GAS_FIELDS = {"nd-ave": abi.FIELD_ND_AVE, "u-ave": abi.FIELD_U_AVE, "v-ave": abi.FIELD_V_AVE,
                  "w-ave": abi.FIELD_W_AVE, "T": abi.FIELD_T, "t1": abi.FIELD_T1, "t2": abi.FIELD_T2,
                  "t3": abi.FIELD_T3, "p": abi.FIELD_P, "mpc": abi.FIELD_MPC}

    def compute_fields(self, T_init=273.15):
        """KineticMaterial.computeFields: dict of the sampled gas fields (ni*nj each)."""
        n = C.c_int64()
        self.d.check(self.d.lib.sf_samples_compute(self.d.ctx, self.sid, float(T_init), C.byref(n)))
        out = {k: self.d.get_field(f, self.sid) for k, f in self.GAS_FIELDS.items()}
        out["num_samples"] = n.value
        return out

    def particle_steps(self):
        """Particle-steps pushed since the species was created."""
        n = C.c_int64()
        self.d.check(self.d.lib.sf_species_particle_steps(self.d.ctx, self.sid, C.byref(n)))
        return n.value

    def get_np(self):
        n = C.c_int64()
        self.d.check(self.d.lib.sf_particles_count(self.d.ctx, self.sid, C.byref(n)))
        return n.value

    def get_den(self):
        return self.d.get_field(abi.FIELD_ND, self.sid)

    def get_count(self):
        return self.d.get_field(abi.FIELD_COUNT, self.sid)

    def get_uvw(self):
        return tuple(self.d.get_field(f, self.sid) for f in (abi.FIELD_U, abi.FIELD_V, abi.FIELD_W))

    def download(self):
        n = self.get_np()
        lc = np.zeros((max(n, 1), 2))
        vel = np.zeros((max(n, 1), 3))
        got = C.c_int64()
        self.d.check(self.d.lib.sf_particles_download(self.d.ctx, self.sid, n, abi.ptr(lc),
                                                      abi.ptr(vel), C.byref(got)))
        return lc[:got.value], vel[:got.value]

    def download_weights(self):
        """mpw of the particles download() returns, in the same order."""
        n = self.get_np()
        w = np.zeros(max(n, 1))
        got = C.c_int64()
        self.d.check(self.d.lib.sf_particles_download_weights(self.d.ctx, self.sid, n, abi.ptr(w), C.byref(got)))
        return w[:got.value]

    def surface_flux(self):
        ns = self.d.spec.seg_xy.reshape(-1, 4).shape[0]
        flux = np.zeros(max(2 * ns, 1))
        dep = np.zeros(max(2 * ns, 1))
        self.d.check(self.d.lib.sf_get_surface_flux(self.d.ctx, self.sid, abi.ptr(flux),
                                                    abi.ptr(dep)))
        return flux[:2 * ns], dep[:2 * ns]


class PoissonSolver:
    """GPU nonlinear Poisson solver with Boltzmann electrons (pic/PoissonSolver.java).

    Arguments follow the <solver type="poisson"> element: n0, Te0 (eV), phi0, eps_r,
    tol (residual target, here on the FP64 nonlinear residual ||R||_2/N), max_it.
    """

    EPS0 = 8.85418782e-12

    def __init__(self, domain: GpuDomain, n0=1e12, Te0=2.0, phi0=0.0, eps_r=1.0, tol=1e-6,
                 max_it=60, cycles=4, linear=False):
        self.d = domain
        self.prm = abi.PoissonParams()
        self.prm.n0, self.prm.kTe0, self.prm.phi0 = n0, Te0, phi0
        self.prm.eps = self.EPS0 * eps_r
        self.prm.tol = tol
        self.prm.max_it = max_it
        self.prm.cycles = cycles
        self.prm.use_learned = 0
        self.prm.linear = 1 if linear else 0

    def update_rho(self):
        """SolverModule.updateRho from the GPU-resident species densities."""
        self.d.check(self.d.lib.sf_update_rho(self.d.ctx))

    def set_bc_values(self, bc):
        bc = np.ascontiguousarray(bc, np.float64)
        self.d.check(self.d.lib.sf_set_bc_values(self.d.ctx, abi.ptr(bc)))

    def solve(self, rho=None, phi=None, check=True):
        """PoissonSolver.update(): returns (phi or None, stats dict)."""
        st = abi.SolveStats()
        rho_a = None if rho is None else np.ascontiguousarray(rho, np.float64)
        phi_a = None if phi is None else np.array(phi, np.float64, copy=True)
        rc = self.d.lib.sf_poisson_nl(self.d.ctx, C.byref(self.prm), abi.ptr(rho_a), abi.ptr(phi_a),
                                      C.byref(st))
        if check:
            self.d.check(rc)
        out = st.as_dict()
        out["status"] = rc
        return phi_a, out

    def update_gradient_field(self, copy=False):
        """PotentialSolver.updateGradientField: E = -grad(phi) on the device."""
        if copy:
            efi = np.zeros(self.d.ni * self.d.nj)
            efj = np.zeros(self.d.ni * self.d.nj)
            self.d.check(self.d.lib.sf_efield(self.d.ctx, abi.ptr(efi), abi.ptr(efj)))
            return efi, efj
        self.d.check(self.d.lib.sf_efield(self.d.ctx, None, None))
        return None

    def boltzmann(self):
        ne = np.zeros(self.d.ni * self.d.nj)
        self.d.check(self.d.lib.sf_boltzmann(self.d.ctx, abi.ptr(ne)))
        return ne

    def use_learned(self, on=True, mode=1):
        """Use the domain's network (LearnedWarmStart must exist): mode 1 starts each solve
        from its predicted potential; mode 2 uses it as a coarse correction inside the
        PCG and trains it on each converged solve's first residual."""
        self.prm.use_learned = int(mode) if on else 0


class LearnedWarmStart:
    """The U-Net warm start of the Poisson solve (no reference counterpart).

    Created on a domain, it learns from every converged solve of that domain while
    training is on; PoissonSolver.use_learned() makes the solves start from its
    prediction.  base: channels of the first level (16 or 32); down: coarsening of the
    network grid relative to the mesh.
    """

    def __init__(self, domain: GpuDomain, base=32, down=4, seed=0, lr=1e-3, iters_per_sample=1):
        self.d = domain
        self.d.check(self.d.lib.sf_unet_init(self.d.ctx, base, down, seed))
        self.Hn, self.Wn = (domain.nj - 1) // down, (domain.ni - 1) // down
        self.train(True, lr, iters_per_sample)

    def train(self, on=True, lr=1e-3, iters_per_sample=1, every=1):
        """Online training on/off; one training pair every `every` converged solves."""
        self.d.check(self.d.lib.sf_unet_set_training(self.d.ctx, int(on), float(lr),
                                                     int(iters_per_sample), int(every)))

    def stats(self):
        loss, n, ms = C.c_double(), C.c_int64(), C.c_double()
        used, rej = C.c_int64(), C.c_int64()
        self.d.check(self.d.lib.sf_unet_stats(self.d.ctx, C.byref(loss), C.byref(n), C.byref(ms),
                                              C.byref(used), C.byref(rej)))
        return {"loss": loss.value, "samples": n.value, "train_ms": ms.value, "used": used.value,
                "rejected": rej.value}

    def tensor_cores(self, on=True):
        """3x3 convolutions on the tcgen05 tensor cores (the default) or on mma.sync."""
        self.d.check(self.d.lib.sf_unet_set_tensor_cores(self.d.ctx, int(on)))

    def tensor_core_convs(self):
        n = C.c_int64()
        self.d.check(self.d.lib.sf_unet_tensor_core_stats(self.d.ctx, C.byref(n)))
        return n.value

    def nparams(self):
        n = C.c_int64()
        self.d.check(self.d.lib.sf_unet_debug(self.d.ctx, None, None, None, None, C.byref(n)))
        return n.value

    def params(self, set_to=None):
        n = self.nparams()
        if set_to is not None:
            p = np.ascontiguousarray(set_to, np.float32)
            assert p.size == n
            self.d.check(self.d.lib.sf_unet_params(self.d.ctx, None, abi.ptr(p)))
            return p
        out = np.zeros(n, np.float32)
        self.d.check(self.d.lib.sf_unet_params(self.d.ctx, abi.ptr(out), None))
        return out

    def forward_backward(self, x, dpred=None):
        """Network output for x (Hn, Wn, 16) and, with dpred, the parameter gradients."""
        x = np.ascontiguousarray(x, np.float32)
        assert x.shape == (self.Hn, self.Wn, 16)
        pred = np.zeros((self.Hn, self.Wn), np.float32)
        grads = None
        n = C.c_int64()
        if dpred is not None:
            dpred = np.ascontiguousarray(dpred, np.float32)
            grads = np.zeros(self.nparams(), np.float32)
        self.d.check(self.d.lib.sf_unet_debug(self.d.ctx, abi.ptr(x), abi.ptr(dpred), abi.ptr(pred),
                                              abi.ptr(grads), C.byref(n)))
        return pred, grads


def _sigma(model, c=(0, 0, 0, 0), diam=0.0, T_ref=273.0, omega=0.5, vss_alpha=1.0):
    s = abi.Sigma()
    s.model = model
    for k in range(4):
        s.c[k] = float(c[k]) if k < len(c) else 0.0
    s.diam, s.T_ref, s.omega, s.vss_alpha = diam, T_ref, omega, vss_alpha
    return s


class DSMC:
    """GPU DSMC pair interaction (collisions/DSMC.java): pair="mat1,mat2" with mat2 the same
    kinetic material (the default) or another one.  The cross-section model and
    coefficients are the interaction's; diam, T_ref, omega and vss_alpha are mat1's, and
    mat2's come in material2_params (a dict with those keys) for two materials."""

    def __init__(self, domain: GpuDomain, material: KineticMaterial, model=4, c=(0, 0, 0, 0), diam=0.0,
                 T_ref=273.0, omega=0.5, vss_alpha=1.0, sig_cr_max=1e-16, frequency=1,
                 material2: KineticMaterial = None, material2_params=None):
        self.d, self.km = domain, material
        self.km2 = material2 if material2 is not None else material
        self.sigma = _sigma(model, c, diam, T_ref, omega, vss_alpha)
        p2 = dict(diam=diam, T_ref=T_ref, omega=omega, vss_alpha=vss_alpha)
        if material2_params:
            p2.update(material2_params)
        self.sigma2 = _sigma(model, c, **p2)
        self.sig_cr_max0 = sig_cr_max
        self.frequency = frequency

    def perform(self, dt, wait=True):
        """DSMC.perform: the number of collisions.  wait=False queues the collisions and
        returns None (the per-cell sums of counts() hold them)."""
        n = C.c_int64()
        self.d.check(self.d.lib.sf_dsmc_pair(self.d.ctx, self.km.sid, self.km2.sid, C.byref(self.sigma),
                                             C.byref(self.sigma2), dt * self.frequency, self.sig_cr_max0,
                                             C.byref(n) if wait else None))
        return n.value if wait else None

    def counts(self):
        nc = (self.d.ni - 1) * (self.d.nj - 1)
        cnt = np.zeros(nc)
        real = np.zeros(nc)
        self.d.check(self.d.lib.sf_dsmc_pair_get_counts(self.d.ctx, self.km.sid, self.km2.sid, abi.ptr(cnt),
                                                        abi.ptr(real)))
        return cnt, real


class MCC:
    """GPU Monte Carlo collisions (collisions/MCC.java) of a kinetic species with a target."""

    def __init__(self, domain: GpuDomain, material: KineticMaterial, target_mass, den, temp, u=None, v=None,
                 w=None, model=0, sigma_model=0, c=(0, 0, 0, 0), diam=0.0, T_ref=273.0, omega=0.5):
        self.d, self.km, self.model = domain, material, model
        self.sigma = _sigma(sigma_model, c, diam, T_ref, omega)
        arr = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (den, u, v, w, temp)]
        self.d.check(self.d.lib.sf_mcc_set_target(self.d.ctx, target_mass, *[abi.ptr(a) for a in arr]))

    def perform(self, dt, product: "KineticMaterial" = None, ionization_energy=None):
        """MCC.perform: the number of collisions.  With model MCC_IONIZATION, `product` is
        the ion species and `ionization_energy` the target's (eV); the return value is then
        (collisions, new electrons, new ions)."""
        n = C.c_int64()
        if self.model == abi.MCC_IONIZATION:
            if product is None or ionization_energy is None:
                raise ValueError("ionization needs the product species and the ionization energy")
            ne, ni = C.c_int64(), C.c_int64()
            self.d.check(self.d.lib.sf_mcc_ionization(self.d.ctx, self.km.sid, product.sid, C.byref(self.sigma),
                                                      float(ionization_energy), dt, C.byref(n), C.byref(ne),
                                                      C.byref(ni)))
            return n.value, ne.value, ni.value
        self.d.check(self.d.lib.sf_mcc(self.d.ctx, self.km.sid, self.model, C.byref(self.sigma), dt,
                                       C.byref(n)))
        return n.value

    def sums(self, reset=False):
        """S (target energy term), count_sum, real_sum and delta_n node fields (ni*nj)."""
        nn = self.d.ni * self.d.nj
        out = {k: np.zeros(nn) for k in ("S", "count_sum", "real_sum", "delta_n")}
        self.d.check(self.d.lib.sf_mcc_get_sums(self.d.ctx, abi.ptr(out["S"]), abi.ptr(out["count_sum"]),
                                                abi.ptr(out["real_sum"]), abi.ptr(out["delta_n"]), int(reset)))
        return out


class GpuBatch:
    """Independent instances advanced together (sf_batch_*): each instance is a GpuDomain
    with one KineticMaterial; a step runs every instance's source, push + scatter (one
    batched device phase) and Poisson solve + E (overlapping on the GPU)."""

    def __init__(self, domains, materials, threads=8):
        self.domains, self.materials = list(domains), list(materials)
        self.lib = abi.load()
        n = len(self.domains)
        ctxs = (C.c_void_p * n)(*[d.ctx.value for d in self.domains])
        sids = np.ascontiguousarray([m.sid for m in self.materials], np.int32)
        h = C.c_void_p()
        rc = self.lib.sf_batch_create(ctxs, abi.ptr(sids), n, int(threads), C.byref(h))
        abi.check(rc, None)
        self.b = h
        self._sids = sids

    def check(self, rc):
        if rc != abi.SF_OK:
            raise abi.SfError(rc, (self.lib.sf_batch_last_error(self.b) or b"").decode())

    def set_source(self, i, seg_xy, den, v_drift, temp):
        seg = np.ascontiguousarray(seg_xy, np.float64).reshape(-1)
        self.check(self.lib.sf_batch_set_source(self.b, int(i), abi.ptr(seg), den, v_drift, temp))

    def step(self, dt, solver: "PoissonSolver"):
        st = abi.BatchStats()
        self.check(self.lib.sf_batch_step(self.b, float(dt), C.byref(solver.prm), C.byref(st)))
        return st.as_dict()

    def tuning(self):
        bps, sb = C.c_int32(), C.c_int32()
        cyc = np.zeros(3, np.int32)
        self.check(self.lib.sf_batch_tuning(self.b, C.byref(bps), C.byref(sb), abi.ptr(cyc)))
        return {"push_blocks_per_sm": bps.value, "slow_blocks_per_sm": sb.value,
                "pcg_iterations_by_bucket": cyc.tolist()}

    def close(self):
        if self.b:
            self.lib.sf_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
