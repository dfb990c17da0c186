"""The learned Poisson warm start: U-Net kernels against a PyTorch CPU reference of the
same network, and what the trained network gains over the plain warm start.

Gradient check: the library's parameters are loaded into a torch model of the same
architecture (3x3 convs + ReLU, 2x2 average pooling, nearest upsampling, concatenated
skips, 1x1 FP32 head), evaluated in float64, that rounds inputs, conv weights, every
stored activation and every stored activation gradient to BF16 where the GPU stores
them.  On dyadic values no FP32 sum rounds, so the two must agree exactly; on random
values they agree to BF16 level (tolerances in each test).

Gain: on the 81x41 electrode mesh the electrode potential follows a sinusoid and rho a
slow modulation; after online training on 300 solves, each of the next solves is run
twice from the same previous potential -- with the learned warm start and plain -- and
both must reach the same residual; the learned start must lower the initial residual.
"""
import numpy as np
import pytest

from starfish_gb300 import abi
from starfish_gb300 import workloads as W

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _bf16(t):
    return t.to(torch.bfloat16).to(t.dtype)


class RoundBF16(torch.autograd.Function):
    """An activation the GPU stores in BF16: its value and its gradient are both rounded."""

    @staticmethod
    def forward(ctx, x):
        return _bf16(x)

    @staticmethod
    def backward(ctx, g):
        return _bf16(g)


class RoundBF16Weight(torch.autograd.Function):
    """The BF16 copy of an FP32 master weight: rounded value, FP32 gradient."""

    @staticmethod
    def forward(ctx, x):
        return _bf16(x)

    @staticmethod
    def backward(ctx, g):
        return g


def unet_reference(params, x, base, levels=4):
    """Forward pass of the library's U-Net in torch; params: list of leaf tensors in the
    library's flattening (conv w [co][ky][kx][ci], conv b, ..., head w, head b)."""
    import torch.nn.functional as F
    C = [base << l for l in range(levels)]
    it = iter(params)

    def conv(h):
        w = next(it)  # (co, 3, 3, ci)
        b = next(it)
        wt = RoundBF16Weight.apply(w).permute(0, 3, 1, 2)
        return RoundBF16.apply(F.relu(F.conv2d(h, wt, b, padding=1)))

    h = RoundBF16.apply(x)
    skips = []
    for l in range(levels):
        h = conv(h)
        h = conv(h)
        if l < levels - 1:
            skips.append(h)
            h = RoundBF16.apply(F.avg_pool2d(h, 2))
    for k in range(levels - 1):
        skip = skips[levels - 2 - k]
        up = F.interpolate(h, scale_factor=2, mode="nearest")
        h = RoundBF16.apply(torch.cat([up, skip], dim=1))
        h = conv(h)
        h = conv(h)
    hw = next(it)
    hb = next(it)
    return (h * hw.view(1, -1, 1, 1)).sum(dim=1)[0] + hb[0]


def _param_shapes(base, levels=4, cin=16):
    C = [base << l for l in range(levels)]
    shapes = []
    c = cin
    for l in range(levels):
        shapes += [(C[l], 3, 3, c), (C[l],), (C[l], 3, 3, C[l]), (C[l],)]
        c = C[l]
    for l in range(levels - 2, -1, -1):
        shapes += [(C[l], 3, 3, C[l + 1] + C[l]), (C[l],), (C[l], 3, 3, C[l]), (C[l],)]
    shapes += [(C[0],), (1,)]
    return shapes


def _split(flat, shapes):
    out, off = [], 0
    for s in shapes:
        n = int(np.prod(s))
        out.append(flat[off:off + n].reshape(s))
        off += n
    assert off == flat.size
    return out


def _compare(net, base, p, x, dpred):
    """GPU forward + backward against the float64 torch reference; returns the forward
    relative error and per-tensor (relative error, cosine) of the parameter gradients."""
    shapes = _param_shapes(base)
    net.params(set_to=p)
    assert np.array_equal(net.params(), p)
    pred, grads = net.forward_backward(x, dpred)
    # float64 reference: CPU fp32 convolutions may take reduced-precision library paths
    tp = [torch.tensor(a.astype(np.float64), requires_grad=True) for a in _split(p, shapes)]
    xt = torch.tensor(x.astype(np.float64)).permute(2, 0, 1).unsqueeze(0)
    out = unet_reference(tp, xt, base)
    ref = out.detach().numpy()
    err = np.linalg.norm(pred - ref) / np.linalg.norm(ref)
    (out * torch.tensor(dpred.astype(np.float64))).sum().backward()
    res = []
    for a, t in zip(_split(grads, shapes), tp):
        a = a.reshape(-1)
        b = t.grad.numpy().reshape(-1)
        nb = np.linalg.norm(b)
        res.append((np.linalg.norm(a - b) / max(nb, 1e-30), float(a @ b / max(np.linalg.norm(a) * nb, 1e-30))))
    return err, res


def _net(base):
    from starfish_gb300.plugin import GpuDomain, LearnedWarmStart
    dom = GpuDomain(W.es_pic_mesh(65, 33, 1e-3))  # network grid 32 x 64
    return dom, LearnedWarmStart(dom, base=base, down=1, seed=5)


@pytest.mark.parametrize("base", [16, 32])
def test_unet_exact_on_dyadic_values(gpulib, base):
    """Sparse +-1 weights (about two nonzero taps per output, so magnitudes stay level),
    integer biases, inputs and output gradients, head weights 1: every value is a small
    multiple of 1/64, no FP32 product or sum rounds, and each stored BF16 value is rounded
    from the same exact number on both sides, so the GPU must match the reference exactly
    and any index or data-flow error shows as a mismatch.  (The same values give identical
    FP32 and FP64 reference results.)"""
    dom, net = _net(base)
    try:
        shapes = _param_shapes(base)
        rng = np.random.default_rng(base + 1)
        parts = []
        for sh in shapes[:-2]:
            if len(sh) == 4:
                nz = rng.random(sh) < 2.0 / (9 * sh[3])
                parts.append(np.where(nz, rng.choice([-1.0, 1.0], sh), 0.0))
            else:
                parts.append(rng.integers(-1, 2, sh).astype(np.float64))
        parts += [np.ones(shapes[-2]), np.zeros(1)]
        p = np.concatenate([a.reshape(-1) for a in parts]).astype(np.float32)
        x = rng.integers(-4, 5, (net.Hn, net.Wn, 16)).astype(np.float32)
        dpred = rng.integers(-3, 4, (net.Hn, net.Wn)).astype(np.float32)
        err, res = _compare(net, base, p, x, dpred)
        assert err <= 1e-7, f"forward relative error {err:.3g}"
        bad = [f"tensor {k} {shapes[k]}: rel {r:.3g}" for k, (r, c) in enumerate(res) if not r <= 1e-7]
        assert not bad, "; ".join(bad)
    finally:
        dom.close()


def test_unet_matches_torch_random(gpulib):
    """Random weights (the library's He initialisation), biases and inputs.  Every BF16
    store turns summation-order differences into occasional one-ulp flips that propagate:
    the same rounding-emulated network evaluated on the CPU in FP32 instead of FP64
    differs by ~5e-3 in the forward and by up to 16 % (cosine down to 0.988) in single
    gradient tensors, and tensor-core accumulation is a third order.  So this is a
    BF16-level bound -- forward 2e-2 relative L2, gradients cosine >= 0.95 and relative
    L2 <= 0.35 -- and exactness is left to the dyadic test."""
    base = 32
    dom, net = _net(base)
    try:
        shapes = _param_shapes(base)
        rng = np.random.default_rng(7)
        parts = _split(net.params().copy(), shapes)
        for k in range(1, len(parts) - 2, 2):
            parts[k][:] = rng.normal(0, 0.05, parts[k].shape)
        parts[-2][:] = rng.normal(0, 0.3, parts[-2].shape)
        parts[-1][:] = 0.1
        p = np.concatenate([a.reshape(-1) for a in parts]).astype(np.float32)
        x = rng.normal(0, 1, (net.Hn, net.Wn, 16)).astype(np.float32)
        dpred = rng.normal(0, 1, (net.Hn, net.Wn)).astype(np.float32)
        err, res = _compare(net, base, p, x, dpred)
        assert err < 2e-2, f"forward relative error {err:.3g}"
        bad = [f"tensor {k} {shapes[k]}: rel {r:.3g} cos {c:.4f}" for k, (r, c) in enumerate(res)
               if not (r <= 0.35 and c >= 0.95)]
        assert not bad, f"forward error {err:.3g}; " + "; ".join(bad)
    finally:
        dom.close()


@pytest.mark.parametrize("base", [16, 32])
def test_unet_tensor_core_path_matches_mma_sync(gpulib, base):
    """The tcgen05 convolutions (TMA loads, tensor-memory accumulators) against the
    mma.sync kernels on the same parameters and inputs.  The 64x32 network grid puts every
    level but the 8x4 one on the tensor-core path (rows of 64, 32 and 16 pixels).  On
    dyadic values both paths are exact, so prediction and gradients must be identical;
    the conv counter shows that the tensor-core path ran."""
    dom, net = _net(base)
    try:
        shapes = _param_shapes(base)
        rng = np.random.default_rng(base + 11)
        parts = []
        for sh in shapes[:-2]:
            if len(sh) == 4:
                nz = rng.random(sh) < 2.0 / (9 * sh[3])
                parts.append(np.where(nz, rng.choice([-1.0, 1.0], sh), 0.0))
            else:
                parts.append(rng.integers(-1, 2, sh).astype(np.float64))
        parts += [np.ones(shapes[-2]), np.zeros(1)]
        p = np.concatenate([a.reshape(-1) for a in parts]).astype(np.float32)
        x = rng.integers(-4, 5, (net.Hn, net.Wn, 16)).astype(np.float32)
        dpred = rng.integers(-3, 4, (net.Hn, net.Wn)).astype(np.float32)
        net.params(set_to=p)
        n0 = net.tensor_core_convs()
        net.tensor_cores(True)
        pred_tc, g_tc = net.forward_backward(x, dpred)
        n1 = net.tensor_core_convs()
        net.tensor_cores(False)
        pred_ms, g_ms = net.forward_backward(x, dpred)
        assert net.tensor_core_convs() == n1
        # forward: 3 levels x 2 encoder convs + 3 decoder levels x 2; backward-data: the same
        assert n1 - n0 >= 12, (n0, n1)
        assert np.array_equal(pred_tc, pred_ms)
        assert np.array_equal(g_tc, g_ms)
        # random values: the two accumulation orders agree to BF16 level
        q = net.params().copy()
        for k, (a, sh) in enumerate(zip(_split(q, shapes), shapes)):
            if len(sh) == 1 and k < len(shapes) - 2:
                a[:] = rng.normal(0, 0.05, sh)
        net.params(set_to=q)
        xr = rng.normal(0, 1, (net.Hn, net.Wn, 16)).astype(np.float32)
        net.tensor_cores(True)
        a_tc, _ = net.forward_backward(xr)
        net.tensor_cores(False)
        a_ms, _ = net.forward_backward(xr)
        assert np.linalg.norm(a_tc - a_ms) <= 1e-2 * np.linalg.norm(a_ms)
    finally:
        dom.close()


def _rho(spec, t, rng):
    """Quasi-neutral ion charge with a slow central modulation and 1 % noise."""
    x = np.arange(spec.ni) * spec.dh[0]
    y = np.arange(spec.nj) * spec.dh[1]
    X, Y = np.meshgrid(x, y)
    Lx, Ly = spec.lengths()
    blob = np.exp(-((X - 0.3 * Lx) ** 2 + (Y - 0.5 * Ly) ** 2) / (2 * (0.15 * Ly) ** 2))
    n = 1e12 * (1 + 0.3 * np.sin(2 * np.pi * t / 150.0) * blob) * (1 + 0.01 * rng.standard_normal(X.shape))
    return (abi_QE * n).reshape(-1)


abi_QE = 1.60217646e-19


def test_learned_warm_start_gain(gpulib):
    from starfish_gb300.plugin import GpuDomain, LearnedWarmStart, PoissonSolver
    spec = W.es_pic_mesh(81, 41, 1e-3)
    electrode = spec.bc_value != 0
    dom = GpuDomain(spec)
    try:
        ps = PoissonSolver(dom, n0=1e12, Te0=2.0, tol=1e-6, max_it=60)
        net = LearnedWarmStart(dom, base=16, down=1, seed=1, lr=2e-3, iters_per_sample=4)
        rng = np.random.default_rng(0)
        bc = spec.bc_value.copy()
        period = 400
        n_train, n_test = 300, 40
        for t in range(n_train):
            bc[electrode] = -100 - 100 * np.cos(2 * np.pi * t / period)
            ps.set_bc_values(bc)
            ps.solve(rho=_rho(spec, t, rng))
        st = net.stats()
        assert st["samples"] == n_train - 1
        net.train(False)
        ps_l, ps_p = [], []
        for t in range(n_train, n_train + n_test):
            phi_prev = dom.get_field(abi.FIELD_PHI)
            rho = _rho(spec, t, rng)
            bc[electrode] = -100 - 100 * np.cos(2 * np.pi * t / period)
            ps.set_bc_values(bc)
            ps.use_learned(True)
            _, sl = ps.solve(rho=rho)
            phi_l = dom.get_field(abi.FIELD_PHI)
            ps.use_learned(False)
            phi_p, sp = ps.solve(rho=rho, phi=phi_prev)
            assert sl["residual"] < 1e-6 and sp["residual"] < 1e-6
            # both converge to the same potential (within what the residual allows)
            dphi = np.max(np.abs(phi_l - phi_p))
            assert dphi < 1e-6 * np.max(np.abs(phi_p)), (t, dphi, sl, sp)
            ps_l.append(sl)
            ps_p.append(sp)
        r_l = np.mean([s["initial_residual"] for s in ps_l])
        r_p = np.mean([s["initial_residual"] for s in ps_p])
        it_l = np.mean([s["newton_it"] for s in ps_l])
        it_p = np.mean([s["newton_it"] for s in ps_p])
        msg = (f"learned warm start: initial residual {r_l:.3g} vs plain {r_p:.3g} "
               f"({r_p / r_l:.1f}x lower); Newton iterations {it_l:.2f} vs {it_p:.2f}; "
               f"training loss {st['loss']:.3g}; {net.stats()}")
        print("\n" + msg)
        # training sums its gradients with FP32 atomics, so the network differs slightly
        # from run to run: the bounds leave room for that
        assert r_l < 0.8 * r_p, msg
        assert it_l <= it_p + 0.25, msg
    finally:
        dom.close()


def test_learned_coarse_correction_in_pcg(gpulib):
    """use_learned = 2: the network, trained online on each converged solve's first
    residual, corrects the first preconditioner application of the first Newton step
    inside the PCG.  The solves still reach the FP64 tolerance and the same potential as plain
    solves from the same start; the 64x32 network grid runs on the tensor-core path."""
    from starfish_gb300.plugin import GpuDomain, LearnedWarmStart, PoissonSolver
    spec = W.es_pic_mesh(65, 33, 1e-3, electrode_halfwidth=4e-3)
    electrode = spec.bc_value != 0
    dom = GpuDomain(spec)
    try:
        ps = PoissonSolver(dom, n0=1e12, Te0=2.0, tol=1e-6, max_it=60)
        net = LearnedWarmStart(dom, base=16, down=1, seed=2, lr=2e-3, iters_per_sample=2)
        ps.use_learned(True, mode=2)
        rng = np.random.default_rng(5)
        bc = spec.bc_value.copy()
        period = 300
        for t in range(150):
            bc[electrode] = -100 - 100 * np.cos(2 * np.pi * t / period)
            ps.set_bc_values(bc)
            _, st = ps.solve(rho=_rho(spec, t, rng))
            assert st["residual"] < 1e-6
        assert net.stats()["samples"] >= 100
        assert net.tensor_core_convs() > 0
        net.train(False)
        for t in range(150, 170):
            phi_prev = dom.get_field(abi.FIELD_PHI)
            rho = _rho(spec, t, rng)
            bc[electrode] = -100 - 100 * np.cos(2 * np.pi * t / period)
            ps.set_bc_values(bc)
            ps.use_learned(True, mode=2)
            _, sl = ps.solve(rho=rho)
            phi_l = dom.get_field(abi.FIELD_PHI)
            ps.use_learned(False)
            phi_p, sp = ps.solve(rho=rho, phi=phi_prev)
            assert sl["residual"] < 1e-6 and sp["residual"] < 1e-6, (sl, sp)
            assert np.max(np.abs(phi_l - phi_p)) < 1e-6 * np.max(np.abs(phi_p))
    finally:
        dom.close()


def test_rejected_prediction_still_converges(gpulib):
    """A prediction worse than the previous potential is rejected (phi reverts to the
    previous solution) and the solve converges from there to the same potential."""
    from starfish_gb300.plugin import GpuDomain, LearnedWarmStart, PoissonSolver
    spec = W.es_pic_mesh(81, 41, 1e-3)
    electrode = spec.bc_value != 0
    dom = GpuDomain(spec)
    try:
        ps = PoissonSolver(dom, n0=1e12, Te0=2.0, tol=1e-6, max_it=60)
        net = LearnedWarmStart(dom, base=16, down=1, seed=1)
        rng = np.random.default_rng(3)
        bc = spec.bc_value.copy()
        for t in range(3):
            bc[electrode] = -100.0 - t
            ps.set_bc_values(bc)
            ps.solve(rho=_rho(spec, t, rng))
        net.train(False)
        p = net.params()
        net.params(set_to=(rng.normal(0, 1.0, p.size)).astype(np.float32))  # garbage network
        phi_prev = dom.get_field(abi.FIELD_PHI)
        bc[electrode] = -103.0
        ps.set_bc_values(bc)
        rho = _rho(spec, 3, rng)
        ps.use_learned(True)
        _, sl = ps.solve(rho=rho)
        st = net.stats()
        assert st["rejected"] == 1 and st["used"] == 0
        phi_l = dom.get_field(abi.FIELD_PHI)
        ps.use_learned(False)
        phi_p, sp = ps.solve(rho=rho, phi=phi_prev)
        assert sl["residual"] < 1e-6, sl
        assert sl["newton_it"] == sp["newton_it"], (sl, sp)
        assert np.max(np.abs(phi_l - phi_p)) < 1e-6 * np.max(np.abs(phi_p))
    finally:
        dom.close()


def test_tensor_core_wait_runs_out_cleanly(gpulib):
    """Failure detection of the tcgen05 pipeline without a fault: a convolution whose
    copies are never issued makes its first mbarrier wait run out (20 ms bound); the CTAs
    must record the timeout, free their tensor memory and return, so that the call reports
    SF_ERR_TIMEOUT and the context keeps working (a tensor-core forward pass afterwards
    matches the mma.sync one)."""
    from starfish_gb300 import abi
    dom, net = _net(16)
    try:
        rc = dom.lib.sf_unet_tensor_core_wait_test(dom.ctx)
        assert rc == abi.SF_ERR_TIMEOUT, rc
        rng = np.random.default_rng(3)
        x = rng.normal(0, 1, (net.Hn, net.Wn, 16)).astype(np.float32)
        n0 = net.tensor_core_convs()
        net.tensor_cores(True)
        a_tc, _ = net.forward_backward(x)
        assert net.tensor_core_convs() > n0
        net.tensor_cores(False)
        a_ms, _ = net.forward_backward(x)
        assert np.linalg.norm(a_tc - a_ms) <= 1e-2 * np.linalg.norm(a_ms)
    finally:
        dom.close()
