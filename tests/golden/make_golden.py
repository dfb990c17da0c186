"""Generates the golden fixtures in this directory from the oracle.

The Java reference ships no tests, golden vectors or fixtures and cannot run here (no
JDK), so the fixtures are produced by the oracle's restatement of the reference
algorithms (oracle/sf_oracle.cpp) on seeded inputs.  Re-run after changing the oracle:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from starfish_gb300 import workloads as W  # noqa: E402

EPS0 = 8.85418782e-12
QE = 1.60217646e-19


def omesh(spec):
    return O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)


def ion_rho(spec, seed, n_mean=1e12):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, spec.ni)
    y = np.linspace(0, 1, spec.nj)
    X, Y = np.meshgrid(x, y)
    n = n_mean * (0.6 + 0.4 * np.cos(2 * np.pi * X) * np.sin(np.pi * Y)) * (1 + 0.05 * rng.standard_normal(X.shape))
    n = n.reshape(-1)
    n[spec.node_type == 0] = 0
    return QE * n


def make_poisson():
    spec = W.es_pic_mesh(81, 41, 1e-3)
    m = omesh(spec)
    rho = ion_rho(spec, 0)
    phi, it, out = O.poisson_nl(m, spec.bc_value, rho, 1e12, 2.0, 0.0, EPS0, np.zeros(spec.nn),
                                max_it=400000, tol=1e-11, nl_max_it=60, nl_tol=1e-9)
    r = O.poisson_residual(m, spec.bc_value, rho, 1e12, 2.0, 0.0, EPS0, phi)
    efi, efj = O.efield(m, phi)
    ne = O.boltzmann(phi, 1e12, 2.0, 0.0)
    np.savez_compressed(os.path.join(HERE, "poisson_es_pic_81x41.npz"), rho=rho, phi=phi, efi=efi,
                        efj=efj, ne=ne, residual=r / spec.nn, newton_it=it)
    print("poisson: NR iterations", it, "residual/N", r / spec.nn)


def make_push():
    spec = W.es_pic_mesh(81, 41, 1e-3)
    ion = W.IonSpecies()
    _, efi, efj = W.electrode_efield(spec)
    efi = efi.astype(np.float32).astype(np.float64)
    efj = efj.astype(np.float32).astype(np.float64)
    pos, vel = W.uniform_maxwellian(spec, ion, 4000, 42)
    lc = np.column_stack([(pos[:, 0] - spec.x0[0]) / spec.dh[0], (pos[:, 1] - spec.x0[1]) / spec.dh[1]])
    i = np.floor(lc)
    lc = i + (lc - i).astype(np.float32).astype(np.float64)
    vel = vel.astype(np.float32).astype(np.float64)
    m = omesh(spec)
    ptr, idx = O.node_segments(m, spec.seg_xy)
    P = np.zeros((lc.shape[0], 12))
    P[:, 0:2] = lc * np.array(spec.dh)
    P[:, 3:6] = vel
    P[:, 6:8] = lc
    P[:, 9] = ion.spwt
    P[:, 10] = 1
    segs = O.seg_table(spec.seg_xy, spec.seg_btype, O.SURF_ABSORB)
    alive, st, flux, dep = O.push(m, efi, efj, ion.charge, ion.mass, 5e-7, segs, ptr, idx, P)
    den = O.update_fields(m, O.node_volumes(m), P)
    np.savez_compressed(os.path.join(HERE, "push_es_pic_81x41.npz"), lc0=lc, vel0=vel, efi=efi, efj=efj,
                        dt=5e-7, alive=P[:, 10].astype(np.int8), lc1=P[:, 6:8], vel1=P[:, 3:6], den=den,
                        stats=st, deposit=dep)
    print("push: survivors", alive, "of", lc.shape[0])


def make_random():
    np.savez_compressed(os.path.join(HERE, "java_random.npz"), seed0=O.jrandom_doubles(0, 16),
                        seed42=O.jrandom_doubles(42, 16), maxw3d_seed7=O.sample_maxw3d(7, 64, 1000.0))


if __name__ == "__main__":
    make_random()
    make_push()
    make_poisson()
