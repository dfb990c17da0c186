"""ctypes front-end of the CPU oracle (``sf_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py``, to check results against and to time the
CPU baseline.  The product never
imports it.  See the header of ``sf_oracle.cpp`` for what is restated and for
the parity status ("parity unpinned" against the Java reference, which has no
tests and cannot run here; pinned by analytic known-answer tests instead).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "sf_oracle.cpp")
_LIB = os.path.join(_HERE, "_build", "libsf_oracle.so")

# Reference codes (core/domain/Mesh.java:107-108, 140-141, 172-173; Boundary.java:124-125)
NODE_OPEN, NODE_DIRICHLET, NODE_INSULATOR, NODE_INTERNAL = -1, 0, 1, 2
DB_OPEN, DB_DIRICHLET, DB_NEUMANN, DB_PERIODIC, DB_SYMMETRY, DB_MESH, DB_SINK = -1, 0, 1, 2, 3, 4, 5
F_RIGHT, F_TOP, F_LEFT, F_BOTTOM = 0, 1, 2, 3
BT_DIRICHLET, BT_OPEN, BT_SINK, BT_VIRTUAL = 0, 1, 2, 3
SURF_PASS, SURF_ABSORB, SURF_NONE, SURF_SPECULAR, SURF_DIFFUSE = -1, 0, 1, 2, 3
DOM_XY, DOM_RZ, DOM_ZR = 0, 1, 2

PARTICLE_FIELDS = 12  # pos[3], vel[3], lc[2], dt, mpw, alive, spare


def build(force: bool = False) -> str:
    """Compile the oracle shared library with g++ (OpenMP for the threaded baseline)."""
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", _SRC, "-o", _LIB]
        subprocess.check_call(cmd)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _declare(_lib)
    return _lib


def _p(dt):
    return np.ctypeslib.ndpointer(dtype=dt, flags="C_CONTIGUOUS")


def _declare(L):
    d, i8, i32, u8 = _p(np.float64), _p(np.int8), _p(np.int32), _p(np.uint8)
    vp = C.c_void_p
    L.orc_jrandom_doubles.argtypes = [C.c_int64, C.c_int, d]
    L.orc_sample_maxw3d.argtypes = [C.c_int64, C.c_int, C.c_double, d]
    L.orc_sample_maxw_speed.argtypes = [C.c_int64, C.c_int, C.c_double, d]
    L.orc_bird_gamma.argtypes = [C.c_double]
    L.orc_bird_gamma.restype = C.c_double
    L.orc_node_volumes.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, d]
    L.orc_cell_volumes.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, d]
    L.orc_node_segments.argtypes = [C.c_int, C.c_int, d, d, C.c_int, d, vp, vp]
    L.orc_node_segments.restype = C.c_int
    L.orc_assemble.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, i32] + [vp] * 10
    L.orc_poisson_nl.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, d, d,
                                 C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_int, C.c_double, C.c_int, C.c_double, d, d]
    L.orc_poisson_nl.restype = C.c_int
    L.orc_poisson_residual.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, d, d,
                                       C.c_double, C.c_double, C.c_double, C.c_double, d, vp]
    L.orc_poisson_residual.restype = C.c_double
    L.orc_efield.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, d, d, d]
    L.orc_boltzmann.argtypes = [C.c_int, d, C.c_double, C.c_double, C.c_double, d]
    L.orc_push.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, d, d, C.c_double,
                           C.c_double, C.c_double, C.c_int, d, i32, i32, C.c_int, d, d, d, d,
                           C.c_int64, C.c_int]
    L.orc_push.restype = C.c_int
    L.orc_update_fields.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, d, C.c_int, d,
                                    C.c_double, d, vp, vp, vp]
    L.orc_update_samples.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, C.c_int, d, d]
    L.orc_compute_fields.argtypes = [C.c_int, d, C.c_int, d, C.c_double, C.c_double, d]
    L.orc_add_particles.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, d, d, C.c_double,
                                    C.c_double, C.c_double, C.c_int, d]
    L.orc_maxwellian_source.argtypes = [C.c_int64, C.c_int, d, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_double, C.c_double, d, C.c_int, d]
    L.orc_maxwellian_source.restype = C.c_int
    L.orc_uniform_source.argtypes = [C.c_int64, C.c_int, d, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_double, d, C.c_int, d]
    L.orc_uniform_source.restype = C.c_int
    i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    L.orc_point_internal.argtypes = [C.c_int, d, i32, C.c_double, C.c_double]
    L.orc_point_internal.restype = C.c_int
    L.orc_preload.argtypes = [C.c_int64, C.c_int, C.c_int, d, d, C.c_int, C.c_int, d, i32, C.c_double, C.c_double,
                              C.c_double, C.c_double, C.c_double, C.c_int, d]
    L.orc_preload.restype = C.c_int
    L.orc_dsmc.argtypes = [C.c_int, C.c_int, d, C.c_int, d, C.c_double, C.c_double, C.c_double,
                           C.c_double, C.c_double, C.c_double, C.c_double, d, d, C.c_int64]
    L.orc_dsmc.restype = C.c_long
    L.orc_dsmc_pair.argtypes = [C.c_int, C.c_int, d, C.c_int, d, C.c_double, C.c_double, C.c_int, d, C.c_double,
                                C.c_double] + [C.c_double] * 9 + [d, d, C.c_int64]
    L.orc_dsmc_pair.restype = C.c_long
    L.orc_mcc.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, C.c_int, d, C.c_double,
                          C.c_double, d, d, d, d, d, C.c_double, C.c_double, C.c_int, C.c_int64]
    L.orc_mcc.restype = C.c_long
    L.orc_mcc_ex.argtypes = [C.c_int, C.c_int, d, d, C.c_int, i8, i8, C.c_int, d, C.c_double,
                             C.c_double, d, d, d, d, d, C.c_double, C.c_double, C.c_int, C.c_int64,
                             C.c_double, C.c_double, C.c_double, C.c_double, d, d, d, d, C.c_long,
                             d, C.POINTER(C.c_long), d, C.POINTER(C.c_long)]
    L.orc_mcc_ex.restype = C.c_long


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class OMesh:
    """Mesh arguments in the form the oracle takes them.

    ``face_type`` is a (4, max(ni, nj)) int8 array in the reference's Face order
    RIGHT, TOP, LEFT, BOTTOM; rows LEFT/RIGHT are indexed by j, TOP/BOTTOM by i.
    """

    def __init__(self, ni, nj, x0, dh, domain, node_type, face_type):
        self.ni, self.nj = int(ni), int(nj)
        self.x0 = _f64(x0)
        self.dh = _f64(dh)
        self.domain = int(domain)
        self.node_type = np.ascontiguousarray(node_type, dtype=np.int8).reshape(-1)
        self.face_type = np.ascontiguousarray(face_type, dtype=np.int8)
        assert self.face_type.shape == (4, max(self.ni, self.nj))
        assert self.node_type.size == self.ni * self.nj

    def args(self):
        return (self.ni, self.nj, self.x0, self.dh, self.domain, self.node_type,
                self.face_type.reshape(-1))


def node_volumes(m: OMesh):
    out = np.zeros(m.ni * m.nj)
    lib().orc_node_volumes(*m.args(), out)
    return out


def cell_volumes(m: OMesh):
    out = np.zeros((m.ni - 1) * (m.nj - 1))
    lib().orc_cell_volumes(*m.args(), out)
    return out


def node_segments(m: OMesh, seg_xy):
    seg_xy = _f64(seg_xy).reshape(-1)
    nseg = seg_xy.size // 4
    n = lib().orc_node_segments(m.ni, m.nj, m.x0, m.dh, nseg, seg_xy, None, None)
    ptr = np.zeros(m.ni * m.nj + 1, np.int32)
    idx = np.zeros(max(n, 1), np.int32)
    lib().orc_node_segments(m.ni, m.nj, m.x0, m.dh, nseg, seg_xy,
                            ptr.ctypes.data, idx.ctypes.data)
    return ptr, idx[:n]


def assemble(m: OMesh):
    """Returns dict of scipy-free CSR triplets for A, Gi, Gj plus the fixed mask."""
    nnz = np.zeros(3, np.int32)
    args = m.args()
    lib().orc_assemble(*args, nnz, *([None] * 10))
    nu = m.ni * m.nj
    out = {}
    bufs = []
    for k in range(3):
        ptr = np.zeros(nu + 1, np.int32)
        col = np.zeros(int(nnz[k]), np.int32)
        val = np.zeros(int(nnz[k]))
        bufs += [ptr, col, val]
    fixed = np.zeros(nu, np.uint8)
    lib().orc_assemble(*args, nnz, *[b.ctypes.data for b in bufs], fixed.ctypes.data)
    for k, name in enumerate(("A", "Gi", "Gj")):
        out[name] = tuple(bufs[3 * k:3 * k + 3])
    out["fixed"] = fixed
    return out


def poisson_nl(m: OMesh, bc_value, rho, n0, kTe0, phi0, eps, phi_init, max_it=5000,
               tol=1e-6, nl_max_it=50, nl_tol=1e-4):
    phi = _f64(phi_init).copy()
    out = np.zeros(2)
    it = lib().orc_poisson_nl(*m.args(), _f64(bc_value), _f64(rho), n0, kTe0, phi0, eps,
                              int(max_it), tol, int(nl_max_it), nl_tol, phi, out)
    return phi, it, out


def poisson_residual(m: OMesh, bc_value, rho, n0, kTe0, phi0, eps, phi, want_vector=False):
    r = np.zeros(m.ni * m.nj) if want_vector else None
    nrm = lib().orc_poisson_residual(*m.args(), _f64(bc_value), _f64(rho), n0, kTe0, phi0, eps,
                                     _f64(phi), None if r is None else r.ctypes.data)
    return (nrm, r) if want_vector else nrm


def efield(m: OMesh, phi):
    efi = np.zeros(m.ni * m.nj)
    efj = np.zeros(m.ni * m.nj)
    lib().orc_efield(*m.args(), _f64(phi), efi, efj)
    return efi, efj


def boltzmann(phi, n0, kTe0, phi0):
    phi = _f64(phi)
    out = np.zeros_like(phi)
    lib().orc_boltzmann(phi.size, phi, n0, kTe0, phi0, out)
    return out


def seg_table(seg_xy, btype, model, vth=0.0, c_rest=1.0, c_accom=1.0):
    """nseg x 9 table: x1, y1, x2, y2, boundary type, surface model, vth, c_rest, c_accom."""
    seg_xy = _f64(seg_xy).reshape(-1, 4)
    n = seg_xy.shape[0]
    t = np.zeros((n, 9))
    t[:, :4] = seg_xy
    t[:, 4] = btype
    t[:, 5] = model
    t[:, 6] = vth
    t[:, 7] = c_rest
    t[:, 8] = c_accom
    return t


def push(m: OMesh, efi, efj, q, mass, dt, segs, node_seg_ptr, node_seg_idx, parts, seed=0,
         threads=1):
    """One ParticleMover pass.  ``parts`` (n x 12) is updated in place."""
    assert parts.dtype == np.float64 and parts.flags.c_contiguous and parts.shape[1] == 12
    segs = _f64(segs).reshape(-1, 9)
    nseg = segs.shape[0]
    stats = np.zeros(6)
    flux = np.zeros(max(2 * nseg, 1))
    dep = np.zeros(max(2 * nseg, 1))
    ptr = np.ascontiguousarray(node_seg_ptr, np.int32)
    idx = np.ascontiguousarray(node_seg_idx if len(node_seg_idx) else np.zeros(1), np.int32)
    alive = lib().orc_push(*m.args(), _f64(efi), _f64(efj), q, mass, dt, nseg,
                           segs.reshape(-1) if nseg else np.zeros(9), ptr, idx,
                           parts.shape[0], parts.reshape(-1), stats, flux, dep, int(seed),
                           int(threads))
    if alive < 0:
        raise RuntimeError("oracle built without OpenMP")
    return alive, stats, flux[:2 * nseg], dep[:2 * nseg]


def update_fields(m: OMesh, node_vol, parts, nd_back=0.0, moments=False):
    nu = m.ni * m.nj
    den = np.zeros(nu)
    U = np.zeros(nu) if moments else None
    V = np.zeros(nu) if moments else None
    W = np.zeros(nu) if moments else None
    lib().orc_update_fields(*m.args(), _f64(node_vol), parts.shape[0], parts.reshape(-1), nd_back,
                            den, *(None if a is None else a.ctypes.data for a in (U, V, W)))
    return (den, U, V, W) if moments else den


def update_samples(m: OMesh, parts, sums=None):
    """KineticMaterial.updateSamples: adds one sample to the 8 running sums (8, ni*nj)."""
    nu = m.ni * m.nj
    if sums is None:
        sums = np.zeros((8, nu))
    lib().orc_update_samples(*m.args(), parts.shape[0], parts.reshape(-1), sums.reshape(-1))
    return sums


def compute_fields(sums, num_samples, node_vol, mass, T_init):
    """KineticMaterial.computeFields: dict of the 10 sampled gas fields."""
    nu = sums.shape[1]
    out = np.zeros((10, nu))
    lib().orc_compute_fields(nu, sums.reshape(-1), int(num_samples), _f64(node_vol), mass, T_init,
                             out.reshape(-1))
    names = ["nd-ave", "u-ave", "v-ave", "w-ave", "T", "t1", "t2", "t3", "p", "mpc"]
    return {k: out[i] for i, k in enumerate(names)}


def add_particles(m: OMesh, efi, efj, q, mass, dt, parts):
    lib().orc_add_particles(*m.args(), _f64(efi), _f64(efj), q, mass, dt, parts.shape[0],
                            parts.reshape(-1))


def maxwellian_source(seed, seg_xy, den, v_drift, temp, mass, spwt, dt, rem=0.0, cap=1 << 20, domain=0):
    r = np.array([rem], np.float64)
    parts = np.zeros((cap, 12))
    n = lib().orc_maxwellian_source(int(seed), int(domain), _f64(seg_xy), den, v_drift, temp, mass, spwt,
                                    dt, r, cap, parts.reshape(-1))
    return parts[:n].copy(), float(r[0])


def uniform_source(seed, seg_xy, mdot, v_drift, mass, spwt, dt, rem=0.0, cap=1 << 20, domain=0):
    """UniformSource on one segment: (particles n x 12, remainder)."""
    r = np.array([rem], np.float64)
    parts = np.zeros((cap, 12))
    n = lib().orc_uniform_source(int(seed), int(domain), _f64(seg_xy), mdot, v_drift, mass, spwt, dt, r, cap,
                                 parts.reshape(-1))
    return parts[:n].copy(), float(r[0])


def point_internal(seg_xy, seg_btype, x, y):
    """BoundaryModule.isInternal for straight segments (n x 4 end points, boundary types)."""
    seg = _f64(np.asarray(seg_xy).reshape(-1))
    bt = np.ascontiguousarray(seg_btype, np.int32)
    return bool(lib().orc_point_internal(len(bt), seg, bt, float(x), float(y)))


def preload(seed, spec, den, temp, mass, spwt, dt, cap=1 << 22):
    """VolumePreloadSource on the mesh of spec (MeshSpec with segments): particles n x 12."""
    parts = np.zeros((cap, 12))
    seg = _f64(np.asarray(spec.seg_xy).reshape(-1)) if len(spec.seg_xy) else np.zeros(4)
    bt = np.ascontiguousarray(spec.seg_btype, np.int32) if len(spec.seg_btype) else np.zeros(1, np.int32)
    n = lib().orc_preload(int(seed), spec.ni, spec.nj, _f64(spec.x0), _f64(spec.dh), int(spec.domain),
                          len(spec.seg_btype), seg, bt, den, temp, mass, spwt, dt, cap, parts.reshape(-1))
    return parts[:n].copy()


def dsmc(ni, nj, cell_vol, parts, mass, spwt, d_ref, T_ref, omega, vss_alpha, delta_t,
         cell_state, counts, seed):
    return lib().orc_dsmc(ni, nj, _f64(cell_vol), parts.shape[0], parts.reshape(-1), mass, spwt,
                          d_ref, T_ref, omega, vss_alpha, delta_t, cell_state.reshape(-1),
                          counts.reshape(-1), int(seed))


def dsmc_pair(ni, nj, cell_vol, parts1, mass1, spwt1, parts2, mass2, spwt2, mat1, mat2, delta_t,
              cell_state, counts, seed):
    """DSMC.collideCell for two materials; mat1/mat2: dicts of diam, T_ref, omega, vss_alpha."""
    for a in (parts1, parts2, cell_state, counts):
        assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return lib().orc_dsmc_pair(ni, nj, _f64(cell_vol), parts1.shape[0], parts1.reshape(-1), mass1, spwt1,
                               parts2.shape[0], parts2.reshape(-1), mass2, spwt2, mat1["diam"], mat2["diam"],
                               mat1["T_ref"], mat2["T_ref"], mat1["omega"], mat2["omega"],
                               mat1.get("vss_alpha", 1.0), mat2.get("vss_alpha", 1.0), delta_t,
                               cell_state.reshape(-1), counts.reshape(-1), int(seed))


def mcc(m: OMesh, parts, src_mass, tgt_mass, tden, tu, tv, tw, tT, sigma, dt, model, seed):
    return lib().orc_mcc(*m.args(), parts.shape[0], parts.reshape(-1), src_mass, tgt_mass,
                         _f64(tden), _f64(tu), _f64(tv), _f64(tw), _f64(tT), sigma, dt,
                         int(model), int(seed))


def mcc_ex(m: OMesh, parts, src_mass, tgt_mass, tden, tu, tv, tw, tT, sigma, dt, model, seed,
           src_spwt=1.0, e_ion=0.0, prod_mass=1.0, prod_spwt=1.0, max_new=0):
    """MCC with every model (2 = ionization) and its outputs: a dict with the collision
    count, the S / count_sum / real_sum / delta_n node fields and the created electrons and
    ions (12-double particles, velocities before the addParticle rewind)."""
    nn = m.ni * m.nj
    out = {k: np.zeros(nn) for k in ("S", "count_sum", "real_sum", "delta_n")}
    new_e = np.zeros((max(max_new, 1), 12))
    new_i = np.zeros((max(max_new, 1), 12))
    ne, ni = C.c_long(), C.c_long()
    out["cols"] = lib().orc_mcc_ex(*m.args(), parts.shape[0], parts.reshape(-1), src_mass, tgt_mass,
                                   _f64(tden), _f64(tu), _f64(tv), _f64(tw), _f64(tT), sigma, dt, int(model),
                                   int(seed), src_spwt, e_ion, prod_mass, prod_spwt, out["S"], out["count_sum"],
                                   out["real_sum"], out["delta_n"], int(max_new), new_e.reshape(-1), C.byref(ne),
                                   new_i.reshape(-1), C.byref(ni))
    out["n_new_e"], out["n_new_i"] = ne.value, ni.value
    out["new_e"] = new_e[:min(ne.value, max_new)]
    out["new_i"] = new_i[:min(ni.value, max_new)]
    return out


def jrandom_doubles(seed, n):
    out = np.zeros(n)
    lib().orc_jrandom_doubles(int(seed), int(n), out)
    return out


def sample_maxw3d(seed, n, v_th):
    out = np.zeros((n, 3))
    lib().orc_sample_maxw3d(int(seed), int(n), v_th, out.reshape(-1))
    return out


def sample_maxw_speed(seed, n, v_th):
    out = np.zeros(n)
    lib().orc_sample_maxw_speed(int(seed), int(n), v_th, out)
    return out


def bird_gamma(x):
    return lib().orc_bird_gamma(float(x))
