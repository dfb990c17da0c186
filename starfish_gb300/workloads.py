"""Synthetic workloads (mesh, boundaries, species, initial particles).

They stand in for the reference's XML decks: an 81x41 ES-PIC case shaped like the
tutorial (dat/examples/tutorial/step2), its 2049x1025 scaled version, an
axisymmetric DSMC jet (dat/examples/DSMC/jet shape) and batches of uneven
ES-PIC instances.  Everything is generated from a seed; no dataset is involved.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi

AMU = 1.66053886e-27   # Constants.AMU (core/common/Constants.java:24)
QE = 1.60217646e-19    # Constants.QE
KB = 1.3806503e-23     # Constants.K
EPS0 = 8.85418782e-12  # Constants.EPS0
EV_TO_K = QE / KB      # Constants.EVtoK


@dataclass
class MeshSpec:
    ni: int
    nj: int
    x0: tuple
    dh: tuple
    domain: int
    node_type: np.ndarray      # int8 ni*nj, j-major
    face_type: np.ndarray      # int8 (4, max(ni,nj))
    bc_value: np.ndarray       # float64 ni*nj
    seg_xy: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))
    seg_btype: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    node_seg_ptr: np.ndarray | None = None
    node_seg_idx: np.ndarray | None = None

    @property
    def nn(self):
        return self.ni * self.nj

    def lengths(self):
        return ((self.ni - 1) * self.dh[0], (self.nj - 1) * self.dh[1])

    def desc(self) -> abi.MeshDesc:
        """ctypes descriptor; the arrays stay owned by this object."""
        if self.node_seg_ptr is None:
            self.node_seg_ptr, self.node_seg_idx = abi.build_node_segments(
                self.ni, self.nj, self.x0, self.dh, self.seg_xy)
        self._keep = [np.ascontiguousarray(self.node_type, np.int8),
                      np.ascontiguousarray(self.face_type, np.int8),
                      np.ascontiguousarray(self.bc_value, np.float64),
                      np.ascontiguousarray(self.seg_xy, np.float64).reshape(-1),
                      np.ascontiguousarray(self.seg_btype, np.int32),
                      np.ascontiguousarray(self.node_seg_ptr, np.int32),
                      np.ascontiguousarray(self.node_seg_idx if len(self.node_seg_idx)
                                           else np.zeros(1), np.int32)]
        d = abi.MeshDesc()
        d.ni, d.nj = self.ni, self.nj
        d.x0[0], d.x0[1] = self.x0
        d.dh[0], d.dh[1] = self.dh
        d.domain_type = self.domain
        d.node_type = self._keep[0].ctypes.data
        d.face_type = self._keep[1].ctypes.data
        d.bc_value = self._keep[2].ctypes.data
        d.node_vol = None
        d.n_segments = int(self.seg_xy.reshape(-1, 4).shape[0])
        d.seg_xy = self._keep[3].ctypes.data
        d.seg_btype = self._keep[4].ctypes.data
        d.node_seg_ptr = self._keep[5].ctypes.data
        d.node_seg_idx = self._keep[6].ctypes.data
        return d


def rectangle_segments(xlo, ylo, xhi, yhi):
    """Closed clockwise path so that LinearSegment normals (-dy, dx) point out of the solid."""
    pts = [(xlo, ylo), (xlo, yhi), (xhi, yhi), (xhi, ylo), (xlo, ylo)]
    return np.array([[*pts[k], *pts[k + 1]] for k in range(4)], np.float64)


def es_pic_mesh(ni=81, nj=41, dh=1e-3, electrode_halfwidth=4.5e-3, phi_electrode=-100.0,
                walls=abi.DB_DIRICHLET) -> MeshSpec:
    """XY mesh with phi = 0 Dirichlet outer walls and a centred square electrode at
    phi_electrode (solid boundary: nodes inside are Dirichlet, its four segments absorb)."""
    nmax = max(ni, nj)
    node_type = np.full((nj, ni), abi.NODE_OPEN, np.int8)
    bc = np.zeros((nj, ni))
    face = np.full((4, nmax), walls, np.int8)
    if walls == abi.DB_DIRICHLET:
        node_type[0, :] = node_type[-1, :] = abi.NODE_DIRICHLET
        node_type[:, 0] = node_type[:, -1] = abi.NODE_DIRICHLET
    Lx, Ly = (ni - 1) * dh, (nj - 1) * dh
    cx, cy = 0.5 * Lx, 0.5 * Ly
    xlo, xhi = cx - electrode_halfwidth, cx + electrode_halfwidth
    ylo, yhi = cy - electrode_halfwidth, cy + electrode_halfwidth
    x = np.arange(ni) * dh
    y = np.arange(nj) * dh
    X, Y = np.meshgrid(x, y)
    tol = 1e-9 * dh
    inside = (X >= xlo - tol) & (X <= xhi + tol) & (Y >= ylo - tol) & (Y <= yhi + tol)
    node_type[inside] = abi.NODE_DIRICHLET
    bc[inside] = phi_electrode
    segs = rectangle_segments(xlo, ylo, xhi, yhi)
    return MeshSpec(ni, nj, (0.0, 0.0), (dh, dh), abi.DOMAIN_XY, node_type.reshape(-1),
                    face, bc.reshape(-1), segs, np.full(4, abi.BT_DIRICHLET, np.int32))


@dataclass
class IonSpecies:
    mass: float = 16 * AMU       # O+
    charge: float = QE
    spwt: float = 5e5
    temp: float = 1000.0         # K
    v_drift: float = 7000.0      # m/s along +x
    den: float = 1e12            # inlet density (m^-3)

    @property
    def v_th(self):
        return np.sqrt(2 * KB * self.temp / self.mass)   # Utils.computeVth


@dataclass
class EsPicConfig:
    """ES-PIC case: the 81x41 tutorial-like case, or its 2049x1025 scaled version."""
    name: str
    mesh: MeshSpec
    ion: IonSpecies
    dt: float
    n0: float = 1e12
    Te0: float = 2.0
    phi0: float = 0.0
    steps: int = 400
    n_particles: int = 0         # preloaded particles (0: source-fed only)


def config0() -> EsPicConfig:
    """81x41, dx = 1 mm, O+ beam from x = 0, Boltzmann electrons, -100 V electrode."""
    return EsPicConfig("es_pic_81x41", es_pic_mesh(81, 41, 1e-3), IonSpecies(), dt=5e-7, steps=400)


def config1(n_particles=64 * 1024 * 1024) -> EsPicConfig:
    """2049x1025, dx = 0.05 mm, 64M preloaded ions.  dt is scaled with dx (2.5e-8 s)
    to keep config0's 3.5 cells of drift per step."""
    m = es_pic_mesh(2049, 1025, 5e-5, electrode_halfwidth=4.5e-3)
    # macroparticle weight chosen so that the ions fill the gas region at config0's
    # plasma density (1e12 m^-3, per metre of depth)
    Lx, Ly = m.lengths()
    gas_area = Lx * Ly - (2 * 4.5e-3) ** 2
    ion = IonSpecies(spwt=1e12 * gas_area / max(n_particles, 1))
    return EsPicConfig("es_pic_2049x1025_64M", m, ion, dt=2.5e-8, steps=1000, n_particles=n_particles)


def uniform_maxwellian(mesh: MeshSpec, ion: IonSpecies, n: int, seed: int):
    """Positions uniform over the gas region (outside the electrode), velocities drifting
    Maxwellian with the reference's sampler variance (v_th*1.2*sqrt(1/2) per component,
    Utils.SampleMaxw3D, core/common/Utils.java:27-57; normal approximation)."""
    rng = np.random.default_rng(seed)
    Lx, Ly = mesh.lengths()
    xlo, ylo = mesh.seg_xy[:, 0].min(), mesh.seg_xy[:, 1].min()
    xhi, yhi = mesh.seg_xy[:, 0].max(), mesh.seg_xy[:, 1].max()
    out = np.empty((n, 3))
    got = 0
    while got < n:
        m = int((n - got) * 1.05) + 16
        x = rng.uniform(0, Lx, m)
        y = rng.uniform(0, Ly, m)
        ok = ~((x > xlo) & (x < xhi) & (y > ylo) & (y < yhi))
        x, y = x[ok][: n - got], y[ok][: n - got]
        out[got:got + x.size, 0] = x + mesh.x0[0]
        out[got:got + x.size, 1] = y + mesh.x0[1]
        got += x.size
    out[:, 2] = 0
    sig = ion.v_th * 1.2 * np.sqrt(0.5)
    vel = rng.normal(0.0, sig, (n, 3))
    vel[:, 0] += ion.v_drift
    return out, vel


def electrode_efield(mesh: MeshSpec, phi_e=-100.0, width=None):
    """A smooth stand-in potential well around the electrode and its E = -grad(phi)
    (central differences inside, one-sided at the walls, like Solver.evaluateGradient).
    Used before a Poisson solve is available."""
    ni, nj = mesh.ni, mesh.nj
    dx, dy = mesh.dh
    x = np.arange(ni) * dx
    y = np.arange(nj) * dy
    X, Y = np.meshgrid(x, y)
    Lx, Ly = mesh.lengths()
    w = width if width is not None else 0.15 * Ly
    phi = phi_e * np.exp(-(((X - Lx / 2) ** 2 + (Y - Ly / 2) ** 2) / (2 * w * w)))
    phi[0, :] = phi[-1, :] = 0
    phi[:, 0] = phi[:, -1] = 0
    efi = -np.gradient(phi, dx, axis=1, edge_order=1)
    efj = -np.gradient(phi, dy, axis=0, edge_order=1)
    return phi.reshape(-1), efi.reshape(-1), efj.reshape(-1)


# ---------------------------------------------------------------------------------------
# axisymmetric DSMC jet (dat/examples/DSMC/jet shape)
# ---------------------------------------------------------------------------------------
@dataclass
class JetConfig:
    name: str
    mesh: MeshSpec
    mass: float
    spwt: float
    inlet: np.ndarray          # inlet segment (x1, y1, x2, y2) on the axis end
    den: float
    temp: float
    v_drift: float
    wall_temp: float
    diam: float
    T_ref: float
    omega: float
    dt: float
    steps: int
    n_particles: int


def jet_mesh(ni=513, nj=257, Lz=0.5, Lr=0.25, r_inlet=5e-3) -> MeshSpec:
    """ZR mesh: z along x (i), r along y (j).  The axis (r = 0) is a symmetry face; the
    inlet face z = 0 (above the inlet), the outer radius and the far end are diffuse
    walls given as boundary segments, whose normals point into the gas."""
    nmax = max(ni, nj)
    face = np.full((4, nmax), abi.DB_OPEN, np.int8)
    face[abi.FACE_BOTTOM, :] = abi.DB_SYMMETRY
    node_type = np.full(ni * nj, abi.NODE_OPEN, np.int8)
    segs = np.array([
        [0.0, Lr, 0.0, r_inlet],   # inlet plane above the opening, normal +z
        [Lz, Lr, 0.0, Lr],         # outer cylinder, normal -r
        [Lz, 0.0, Lz, Lr],         # far end, normal -z
    ])
    return MeshSpec(ni, nj, (0.0, 0.0), (Lz / (ni - 1), Lr / (nj - 1)), abi.DOMAIN_ZR, node_type, face,
                    np.zeros(ni * nj), segs, np.full(3, abi.BT_DIRICHLET, np.int32))


def config2(n_particles=16 * 1024 * 1024) -> JetConfig:
    """Argon jet: inlet r < 5 mm at 1e22 m^-3, 300 K, 500 m/s; diffuse walls at 300 K; VHS
    (d = 4.17e-10 m, omega = 0.81, T_ref = 273 K); dt = 1e-6 s."""
    m = jet_mesh()
    mass = 40 * AMU
    # weight: the preloaded plume (jet_particles) holds n_particles macroparticles
    spwt = _jet_content(m, 1e22, 5e-3) / n_particles
    return JetConfig("dsmc_jet_513x257_zr", m, mass, spwt, np.array([0.0, 5e-3, 0.0, 0.0]), 1e22, 300.0,
                     500.0, 300.0, 4.17e-10, 273.0, 0.81, 1e-6, 2000, n_particles)


def _jet_density(z, r, n_inlet, r_inlet):
    """Free-jet plume shape used to preload the domain: n_inlet r_in^2 / (r_in^2 + z^2 + r^2),
    with a floor of 1e-4 n_inlet."""
    return n_inlet * np.maximum(r_inlet ** 2 / (r_inlet ** 2 + z ** 2 + r ** 2), 1e-4)


def _jet_content(m: MeshSpec, n_inlet, r_inlet, samples=400):
    Lz, Lr = m.lengths()
    z = (np.arange(samples) + 0.5) * Lz / samples
    r = (np.arange(samples) + 0.5) * Lr / samples
    Z, R = np.meshgrid(z, r)
    dV = 2 * np.pi * R * (Lz / samples) * (Lr / samples)
    return float((_jet_density(Z, R, n_inlet, r_inlet) * dV).sum())


def jet_particles(cfg: JetConfig, n, seed):
    """n macroparticles distributed like the plume: each mesh cell receives a share of
    n proportional to its content (plume density at the cell centre x the cell's volume of
    revolution), positions uniform in z and in area of revolution (r^2) inside the cell;
    drifting Maxwellian velocities at the inlet temperature, radial outflow from the inlet."""
    rng = np.random.default_rng(seed)
    m = cfg.mesh
    dz, dr = m.dh
    z0 = np.arange(m.ni - 1) * dz
    r0 = np.arange(m.nj - 1) * dr
    Z, R = np.meshgrid(z0 + 0.5 * dz, r0 + 0.5 * dr)
    vol = np.pi * ((R + 0.5 * dr) ** 2 - (R - 0.5 * dr) ** 2) * dz
    w = (_jet_density(Z, R, cfg.den, 5e-3) * vol).ravel()
    cells = rng.choice(w.size, size=n, p=w / w.sum())
    ci, cj = cells % (m.ni - 1), cells // (m.ni - 1)
    out = np.empty((n, 3))
    out[:, 0] = z0[ci] + dz * rng.uniform(0, 1, n)
    ra, rb = r0[cj], r0[cj] + dr
    out[:, 1] = np.sqrt(ra ** 2 + (rb ** 2 - ra ** 2) * rng.uniform(0, 1, n))
    out[:, 2] = 0.0
    vth = np.sqrt(2 * KB * cfg.temp / cfg.mass)
    vel = rng.normal(0.0, vth * 1.2 * np.sqrt(0.5), (n, 3))
    rr = np.sqrt(out[:, 0] ** 2 + out[:, 1] ** 2) + 1e-12
    vel[:, 0] += cfg.v_drift * out[:, 0] / rr
    vel[:, 1] += cfg.v_drift * out[:, 1] / rr
    return out, vel


# ---------------------------------------------------------------------------------------
# batched uneven instances (config-0-type cases of many sizes)
# ---------------------------------------------------------------------------------------
@dataclass
class BatchCase:
    mesh: MeshSpec
    ion: IonSpecies
    n_particles: int
    phi_electrode: float
    seed: int


def config4(n_instances=256, seed=0, max_particles=2_000_000, min_particles=10_000):
    """Independent 81x41-type ES-PIC cases: mesh sizes log-uniform from 33x17 to 257x129
    nodes (rounded to 16k + 1 nodes per direction so that multigrid coarsens them), dx = 1
    mm, centred electrode box at a potential uniform in [-200, -20] V, preloaded ion counts
    log-uniform in [1e4, 2e6] at the 1e12 m^-3 plasma density, O+ inlet on the x = 0 face,
    seeds 0..n-1."""
    rng = np.random.default_rng(seed)
    cases = []
    for k in range(n_instances):
        e = rng.uniform(0.0, 3.0)
        ni = int(16 * round(2 * 2 ** e)) + 1
        nj = (ni - 1) // 2 + 1
        phi = rng.uniform(-200.0, -20.0)
        m = es_pic_mesh(ni, nj, 1e-3, electrode_halfwidth=4.5e-3, phi_electrode=phi)
        n = int(round(np.exp(rng.uniform(np.log(min_particles), np.log(max_particles)))))
        Lx, Ly = m.lengths()
        gas_area = Lx * Ly - (2 * 4.5e-3) ** 2
        ion = IonSpecies(spwt=1e12 * gas_area / n)
        cases.append(BatchCase(m, ion, n, phi, k))
    return cases
