"""DSMC on the GPU (sf_dsmc, sf_dsmc_pair) against the reference's candidate draw and the
oracle's DSMC.collideCell.

The reference draws each candidate pair of a cell as p1 uniform and p2 != p1 uniform over
the cell's particle list (collisions/DSMC.java:314-320; one particle of each list for two
materials).  The GPU collides a round of disjoint pairs in parallel; these tests check
that every pair of list positions is still an equally likely candidate, then compare
collision counts and relaxation with the oracle for one and two materials, in ordinary
cells and in the dense cells that the block-per-cell kernel takes."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

AMU = 1.66053886e-27
KB = 1.3806503e-23
ARGON = dict(diam=4.17e-10, T_ref=273.0, omega=0.81, vss_alpha=1.0)
HELIUM = dict(diam=2.33e-10, T_ref=273.0, omega=0.66, vss_alpha=1.0)


def box_mesh(n, dh=1e-3):
    """XY box, all faces symmetry, no segments."""
    spec = W.es_pic_mesh(n, n, dh, walls=abi.DB_SYMMETRY, electrode_halfwidth=1e-12)
    spec.seg_xy = np.zeros((0, 4))
    spec.seg_btype = np.zeros(0, np.int32)
    spec.node_type[:] = abi.NODE_OPEN
    spec.bc_value[:] = 0
    return spec


def per_cell_particles(spec, npc, rng):
    """npc particles uniform in every cell, in cell order."""
    nc1 = spec.ni - 1
    ij = np.repeat(np.arange(nc1 * nc1), npc)
    lc = np.column_stack([ij % nc1, ij // nc1]).astype(np.float64)
    lc += rng.uniform(0.05, 0.95, lc.shape).astype(np.float32).astype(np.float64)
    return lc


def _key(vel):
    v = vel.astype(np.float32)
    b = v.view(np.uint32).astype(np.uint64)
    return (b[:, 0] << np.uint64(32)) | b[:, 1]


def _slot_in_cell(lc, ni):
    cell = np.floor(lc[:, 1]).astype(np.int64) * (ni - 1) + np.floor(lc[:, 0]).astype(np.int64)
    order = np.argsort(cell, kind="stable")
    cs = cell[order]
    first = np.searchsorted(cs, cs, side="left")
    rank = np.empty_like(cell)
    rank[order] = np.arange(cell.size) - first
    return cell, rank


@pytest.mark.parametrize("npc", [4, 6, 8, 9, 64])
def test_dsmc_candidate_pairs_uniform(gpulib, npc):
    """One candidate per cell per call (nsel = 1.001 with sigma g the same for every pair,
    so every candidate collides): the two particles whose velocities changed are the
    candidate, located by their positions in the cell's slot range after the call's cell
    binning.  Over many cells and calls every unordered pair of positions must be drawn
    with equal probability: each of the C(np, 2) counts within 5 binomial sigma of the
    mean, none zero."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, DSMC
    n = 41 if npc == 64 else 33
    spec = box_mesh(n)
    rng = np.random.default_rng(npc)
    lc = per_cell_particles(spec, npc, rng)
    vel = rng.normal(0, 300.0, (lc.shape[0], 3)).astype(np.float32).astype(np.float64)
    assert np.unique(_key(vel)).size == vel.shape[0]
    mass, c0, dt = 40 * AMU, 1e-16, 1e-6
    V = spec.dh[0] * spec.dh[1]
    spwt = 2.0 * 1.001 * V / (npc * npc * dt * c0)  # nsel_f = 1.001 per cell and call
    npairs = npc * (npc - 1) // 2
    calls = max(12, int(math.ceil(200.0 * npairs / (n - 1) ** 2)))
    counts = np.zeros((npc, npc), np.int64)
    drawn = skipped = 0
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, mass, 0.0, spwt, capacity=lc.shape[0] + 16)
        km.add_particles_lc(lc, vel)
        ds = DSMC(dom, km, model=abi.SIGMA_INV, c=[c0, 0, 0, 0], sig_cr_max=c0)
        _, v_before = km.download()
        for _ in range(calls):
            ds.perform(dt)
            lc_a, v_after = km.download()
            cell, rank = _slot_in_cell(lc_a, spec.ni)
            changed = ~np.isin(_key(v_after), _key(v_before))
            ch_cells = cell[changed]
            uc, cnt = np.unique(ch_cells, return_counts=True)
            two = uc[cnt == 2]
            skipped += int((cnt != 2).sum())
            sel = changed & np.isin(cell, two)
            order = np.argsort(cell[sel], kind="stable")
            r = rank[sel][order].reshape(-1, 2)
            lo, hi = r.min(axis=1), r.max(axis=1)
            np.add.at(counts, (lo, hi), 1)
            drawn += r.shape[0]
            v_before = v_after
    finally:
        dom.close()
    assert skipped < 0.01 * drawn
    iu = np.triu_indices(npc, 1)
    c = counts[iu]
    assert c.sum() == drawn and counts[np.tril_indices(npc)].sum() == 0
    p = 1.0 / npairs
    mean = drawn * p
    sd = math.sqrt(drawn * p * (1 - p))
    assert c.min() > 0
    assert np.all(np.abs(c - mean) < 5 * sd), (c.min(), c.max(), mean, sd)
    # the position of a pair's first particle is uniform too (each position is in
    # np - 1 of the C(np, 2) pairs)
    per_slot = counts.sum(axis=0) + counts.sum(axis=1)
    ps = 2.0 / npc
    assert np.all(np.abs(per_slot - drawn * ps) < 5 * math.sqrt(drawn * ps * (1 - ps)))


def _temps(vel, mass):
    v = vel - vel.mean(axis=0)
    return mass * (v ** 2).mean(axis=0) / KB


def _parts(lc, vel, w):
    P = np.zeros((lc.shape[0], 12))
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = w
    P[:, 10] = 1
    return P


def _gas(spec, n, rng, T, mass):
    L = spec.ni - 1
    lc = rng.uniform(0, L, (n, 2))
    lc = np.floor(lc) + (lc - np.floor(lc)).astype(np.float32).astype(np.float64)
    sig = np.sqrt(KB * np.asarray(T, float) / mass)
    vel = (rng.standard_normal((n, 3)) * sig).astype(np.float32).astype(np.float64)
    return lc, vel


def _run_pair(spec, n1, n2, w1, w2, dt, steps, seed, T1=(900.0, 200.0, 200.0), T2=(300.0, 300.0, 300.0)):
    """Argon (anisotropic, hot in x) with helium: the GPU pair interaction and the oracle
    from the same start.  Returns per-step collision counts and species temperatures."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, DSMC
    m1, m2 = 40 * AMU, 4 * AMU
    rng = np.random.default_rng(seed)
    lc1, v1 = _gas(spec, n1, rng, T1, m1)
    lc2, v2 = _gas(spec, n2, rng, T2, m2)
    g = {"cols": [], "T1": [], "T2": []}
    dom = GpuDomain(spec)
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        ka = KineticMaterial(dom, m1, 0.0, w1, capacity=n1 + 16)
        kb = KineticMaterial(dom, m2, 0.0, w2, capacity=n2 + 16)
        ka.add_particles_lc(lc1, v1)
        kb.add_particles_lc(lc2, v2)
        ds = DSMC(dom, ka, model=abi.SIGMA_BIRD463, material2=kb, material2_params=HELIUM, **ARGON)
        for _ in range(steps):
            g["cols"].append(ds.perform(dt))
            g["T1"].append(_temps(ka.download()[1], m1))
            g["T2"].append(_temps(kb.download()[1], m2))
        cnt, real = ds.counts()
        g["count_sum"], g["real_sum"] = cnt, real
        g["v1_end"], g["v2_end"] = ka.download()[1], kb.download()[1]
    finally:
        dom.close()
    P1, P2 = _parts(lc1, v1, w1), _parts(lc2, v2, w2)
    om = _om(spec)
    cv = O.cell_volumes(om)
    nc = (spec.ni - 1) * (spec.nj - 1)
    state = np.zeros((nc, 2))
    state[:, 0] = 1e-16
    counts = np.zeros((nc, 2))
    o = {"cols": [], "T1": [], "T2": []}
    for k in range(steps):
        o["cols"].append(O.dsmc_pair(spec.ni, spec.nj, cv, P1, m1, w1, P2, m2, w2, ARGON, HELIUM, dt, state,
                                     counts, 100 + k))
        o["T1"].append(_temps(P1[:, 3:6], m1))
        o["T2"].append(_temps(P2[:, 3:6], m2))
    o["count_sum"] = counts[:, 0]
    for d in (g, o):
        for k in ("cols", "T1", "T2"):
            d[k] = np.asarray(d[k], float)
    g["start"] = (v1, v2)
    return g, o


def _om(spec):
    return O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)


@pytest.mark.parametrize("ratio", [1.0, 0.25])
def test_dsmc_two_species_matches_oracle(gpulib, ratio):
    """Argon and helium in a 20x20-cell box (sf_dsmc_pair): per-step collision counts, the
    argon anisotropy and the approach of the two temperatures agree with the oracle's
    DSMC.collideCell + ModelElastic (mat1 != mat2).  Equal weights conserve the
    mass-weighted momentum and the energy collision by collision; with w2 = w1 / 4 the
    Boyd update does so only on average, and the counts follow the reference's nsel."""
    spec = box_mesh(21)
    w1 = 1.5e12 if ratio == 1.0 else 3.0e11
    g, o = _run_pair(spec, 30000, 20000, w1, w1 * ratio, 1e-5, 12, seed=7 if ratio == 1.0 else 8)
    gc, oc = g["cols"][2:], o["cols"][2:]
    assert gc.mean() == pytest.approx(oc.mean(), rel=0.05)
    assert g["count_sum"].sum() == g["cols"].sum()
    assert g["real_sum"].sum() == pytest.approx(g["cols"].sum() * 0.5 * w1 * (1 + ratio), rel=1e-12)
    # argon's x-y anisotropy and the argon-helium temperature gap relax alike
    ga, oa = g["T1"][:, 0] - g["T1"][:, 1], o["T1"][:, 0] - o["T1"][:, 1]
    if ratio == 1.0:
        assert ga[-1] < 0.6 * ga[0]
    assert np.allclose(ga, oa, rtol=0.15, atol=20.0)
    gd = g["T1"].mean(axis=1) - g["T2"].mean(axis=1)
    od = o["T1"].mean(axis=1) - o["T2"].mean(axis=1)
    assert np.allclose(gd, od, rtol=0.15, atol=20.0)
    if ratio == 1.0:
        m1, m2 = 40 * AMU, 4 * AMU
        v1, v2 = g["start"]
        p0 = m1 * v1.sum(axis=0) + m2 * v2.sum(axis=0)
        p1 = m1 * g["v1_end"].sum(axis=0) + m2 * g["v2_end"].sum(axis=0)
        scale = m1 * np.abs(v1).sum(axis=0) + m2 * np.abs(v2).sum(axis=0)
        assert np.all(np.abs(p1 - p0) <= 1e-4 * scale)
        e0 = m1 * (v1 ** 2).sum() + m2 * (v2 ** 2).sum()
        e1 = m1 * (g["v1_end"] ** 2).sum() + m2 * (g["v2_end"] ** 2).sum()
        assert e1 == pytest.approx(e0, rel=1e-5)


def test_dsmc_dense_cells_match_oracle(gpulib):
    """Cells of 6000 particles with about 4000 candidates per step go to the
    block-per-cell kernel (over 1024 candidates).  One material: the collision counts and
    the relaxation of an anisotropic temperature agree with the oracle, energy is kept.
    Two materials in the same dense cells: counts and temperatures agree as well."""
    from starfish_gb300.plugin import GpuDomain, KineticMaterial, DSMC
    spec = box_mesh(3)  # 4 cells
    n, mass, dt = 24000, 40 * AMU, 1e-5
    rng = np.random.default_rng(21)
    lc, vel = _gas(spec, n, rng, (900.0, 200.0, 200.0), mass)
    spwt = 2.2e10
    dom = GpuDomain(spec)
    g_cols, g_T = [], []
    try:
        dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
        km = KineticMaterial(dom, mass, 0.0, spwt, capacity=n + 16)
        km.add_particles_lc(lc, vel)
        ds = DSMC(dom, km, model=abi.SIGMA_BIRD463, **ARGON)
        for _ in range(10):
            g_cols.append(ds.perform(dt))
            g_T.append(_temps(km.download()[1], mass))
        v_end = km.download()[1]
    finally:
        dom.close()
    P = _parts(lc, vel, spwt)
    cv = O.cell_volumes(_om(spec))
    state = np.zeros((4, 2))
    state[:, 0] = 1e-16
    counts = np.zeros((4, 2))
    o_cols, o_T = [], []
    for k in range(10):
        o_cols.append(O.dsmc(spec.ni, spec.nj, cv, P, mass, spwt, ARGON["diam"], 273.0, 0.81, 1.0, dt, state,
                             counts, 50 + k))
        o_T.append(_temps(P[:, 3:6], mass))
    g_cols, o_cols = np.array(g_cols[2:], float), np.array(o_cols[2:], float)
    assert o_cols.mean() / 4 > 1024 * 0.25  # about 0.3 of the candidates collide: well above 1024 per cell
    assert g_cols.mean() == pytest.approx(o_cols.mean(), rel=0.05)
    g_T, o_T = np.array(g_T), np.array(o_T)
    ga, oa = g_T[:, 0] - g_T[:, 1], o_T[:, 0] - o_T[:, 1]
    assert ga[-1] < 0.5 * ga[0]
    assert np.allclose(ga, oa, rtol=0.15, atol=20.0)
    assert (v_end ** 2).sum() == pytest.approx((vel ** 2).sum(), rel=1e-5)
    # two materials, dense: 3000 argon + 3000 helium per cell
    g, o = _run_pair(spec, 12000, 12000, 1.5e10, 1.5e10, dt, 8, seed=22)
    assert o["cols"][2:].mean() / 4 > 1024 * 0.25
    assert g["cols"][2:].mean() == pytest.approx(o["cols"][2:].mean(), rel=0.05)
    gd = g["T1"].mean(axis=1) - g["T2"].mean(axis=1)
    od = o["T1"].mean(axis=1) - o["T2"].mean(axis=1)
    assert np.allclose(gd, od, rtol=0.15, atol=20.0)
