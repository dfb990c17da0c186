"""Species change at surfaces (SurfaceInteraction.java specular and cosine handlers with a
product material) on the GPU.

Ions start left of the electrode box of the ES-PIC mesh, moving +x fast enough that every
one crosses the box's left face within one push (no field).  With a product species set
on the box's segments:
- specular: every ion leaves and one product per ion starts at its hit point on the face
  with the reflected velocity of the reference's handler, v + n sqrt(2) |v_xy| (at normal
  incidence (1 - sqrt(2)) v, not the mirror image);
- diffuse with a weight ratio of 2: exactly two products per ion, Maxwellian speeds at the
  product's wall temperature (mean 2/sqrt(pi) vth), cosine-law directions away from the
  face (mean normal cosine 2/3);
- a product species without room makes the push return SF_ERR_OOM.
"""
import numpy as np
import pytest

from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

AMU = 1.66053886e-27
QE = 1.602e-19


def _setup(n, spwt_ion, spwt_prod, model, vth_prod, prod_cap):
    from starfish_gb300.plugin import GpuDomain, KineticMaterial
    spec = W.es_pic_mesh(81, 41, 1e-3)  # box x in [35.5, 44.5] mm, y in [15.5, 24.5] mm
    dom = GpuDomain(spec)
    dom.set_efield(np.zeros(spec.nn), np.zeros(spec.nn))
    ion = KineticMaterial(dom, 16 * AMU, QE, spwt_ion, capacity=n + 16)
    neu = KineticMaterial(dom, 16 * AMU, 0.0, spwt_prod, capacity=prod_cap)
    for s in range(len(spec.seg_btype)):
        ion.set_surface(s, model, vth=vth_prod if model == abi.SURF_DIFFUSE else 0.0, c_rest=1.0, c_accom=1.0)
        ion.set_surface_product(s, neu, vth_prod)
    rng = np.random.default_rng(8)
    lc = np.empty((n, 2))
    lc[:, 0] = rng.uniform(33.0, 35.0, n)
    lc[:, 1] = rng.uniform(17.0, 23.0, n)
    lc = np.floor(lc) + (lc - np.floor(lc)).astype(np.float32).astype(np.float64)
    vel = np.zeros((n, 3))
    vel[:, 0] = 8000.0
    ion.add_particles_lc(lc, vel)
    return spec, dom, ion, neu, lc


def test_specular_product_at_hit_point(gpulib):
    n = 20000
    spec, dom, ion, neu, lc0 = _setup(n, 1e6, 1e6, abi.SURF_SPECULAR, 0.0, n + 16)
    try:
        ion.update_fields(5e-7, stats=False)
        assert ion.get_np() == 0 and neu.get_np() == n
        lc, vel = neu.download()
        assert np.allclose(vel[:, 0], 8000.0 * (1 - np.sqrt(2.0)), rtol=1e-6) and np.all(vel[:, 1:] == 0)
        x = lc[:, 0] * 1e-3
        assert np.all((x > 0.0355 - 1e-6) & (x <= 0.0355))
        assert np.allclose(np.sort(lc[:, 1]), np.sort(lc0[:, 1]), atol=1e-5)
    finally:
        dom.close()


def test_diffuse_product_two_per_hit_cosine_law(gpulib):
    n = 20000
    vth = np.sqrt(2 * 1.3806503e-23 * 300.0 / (16 * AMU))
    spec, dom, ion, neu, _ = _setup(n, 2e6, 1e6, abi.SURF_DIFFUSE, vth, 2 * n + 16)
    try:
        ion.update_fields(5e-7, stats=False)
        assert ion.get_np() == 0 and neu.get_np() == 2 * n
        _, vel = neu.download()
        speed = np.linalg.norm(vel, axis=1)
        assert abs(speed.mean() / (2 / np.sqrt(np.pi) * vth) - 1) < 0.02
        assert np.all(vel[:, 0] <= 0)  # away from the left face (outward normal -x)
        cos_n = -vel[:, 0] / speed
        assert abs(cos_n.mean() - 2 / 3) < 0.01
    finally:
        dom.close()


def test_product_capacity_overflow(gpulib):
    n = 5000
    spec, dom, ion, neu, _ = _setup(n, 1e6, 1e6, abi.SURF_SPECULAR, 0.0, 1000)
    try:
        with pytest.raises(abi.SfError) as e:
            ion.update_fields(5e-7, stats=False)
        assert e.value.code == abi.SF_ERR_OOM
        assert neu.get_np() == 1000
    finally:
        dom.close()
