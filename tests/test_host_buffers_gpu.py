"""Pinned host buffers: sf_set_efield reads them and sf_get_field writes them directly from
kernels; the results must equal those of ordinary (pageable) host arrays, which go through
copies."""
import numpy as np
import pytest

from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _pinned(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()


def test_pinned_and_pageable_host_buffers_agree(gpulib):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(129, 65, 1e-3, walls=abi.DB_OPEN)
    spec.seg_xy = np.zeros((0, 4))
    spec.seg_btype = np.zeros(0, np.int32)
    spec.node_type[:] = abi.NODE_OPEN
    spec.bc_value[:] = 0.0
    rng = np.random.default_rng(9)
    efi = rng.normal(0, 300, spec.nn)
    efj = rng.normal(0, 300, spec.nn)
    n = 50_000
    lc = np.column_stack([rng.uniform(1, spec.ni - 2, n), rng.uniform(1, spec.nj - 2, n)])
    vel = rng.normal(0, 1500.0, (n, 3))
    out = []
    for pinned in (False, True):
        dom = GpuDomain(spec)
        try:
            ei, ej = (_pinned(efi), _pinned(efj)) if pinned else (efi.copy(), efj.copy())
            dom.check(dom.lib.sf_set_efield(dom.ctx, abi.ptr(ei), abi.ptr(ej)))
            km = KineticMaterial(dom, 16 * 1.6605e-27, 1.602e-19, 1e5, capacity=n + 64)
            km.set_sort_interval(0)
            km.add_particles_lc(lc, vel)
            for _ in range(3):
                km.update_fields(1e-7, stats=False)
            nd = _pinned(np.full(spec.nn, -1.0)) if pinned else np.full(spec.nn, -1.0)
            dom.check(dom.lib.sf_get_field(dom.ctx, abi.FIELD_ND, km.sid, abi.ptr(nd)))
            out.append((np.array(nd), km.download()))
        finally:
            dom.close()
    (nd0, (lc0, v0)), (nd1, (lc1, v1)) = out
    assert nd0.max() > 0
    assert np.array_equal(nd0, nd1)
    assert np.array_equal(lc0, lc1) and np.array_equal(v0, v1)
