"""Adjoint of the pair force and of the RK4 rollout (needs a GB300).

* the VJP kernel against torch autograd through a dense FP64 torch
  restatement of the same forces;
* the rollout gradient (checkpointed recomputation) against central finite
  differences (relative step 1e-6) and against the FP64 torch-autograd
  gradient of the same rollout.
Clouds are small enough that every pair stays inside the cutoff, so no pair
crosses kappa*r = 10 (where the force jumps and differences are meaningless).
"""
import numpy as np
import pytest

from demon_simulation_code_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from demon_simulation_code_gb300.adjoint import AdjointKernels  # noqa: E402

C = 1.0 / (4.0 * np.pi * 8.8541878e-12)


def clouds(ns, radius=6e-4, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for n in ns:
        x, y = W.uniform_disk_minsep(rng, n, radius, 1e-4)
        out.append((x, y, rng.normal(0, 1e-4, n), rng.normal(0, 1e-4, n)))
    return out


def torch_forces(x, y, vx, vy, q, m, kappa, kc, gamma, ns):
    fxs, fys = [], []
    off = 0
    for c, n in enumerate(ns):
        xs, ys, qs = x[off:off + n], y[off:off + n], q[off:off + n]
        dx = xs[:, None] - xs[None, :]
        dy = ys[:, None] - ys[None, :]
        eye = torch.eye(n, dtype=torch.bool, device=x.device)
        r = torch.sqrt(torch.where(eye, torch.ones_like(dx), dx * dx + dy * dy))
        a = r * kappa[c]
        mask = (a < 10.0) & ~eye
        g = torch.where(mask, C * qs[:, None] * qs[None, :] * (1 + a) * torch.exp(-a) / r**3,
                        torch.zeros_like(r))
        fx = (g * dx).sum(1) + qs * kc[c] * xs - gamma * m[off:off + n] * vx[off:off + n]
        fy = (g * dy).sum(1) + qs * kc[c] * ys - gamma * m[off:off + n] * vy[off:off + n]
        fxs.append(fx)
        fys.append(fy)
        off += n
    return torch.cat(fxs), torch.cat(fys)


@pytest.fixture(scope="module")
def setup(gpu_ctx):
    from demon_simulation_code_gb300.adjoint import AdjointKernels

    ns = [37, 64, 9]
    data = clouds(ns)
    cat = [torch.tensor(np.concatenate([d[k] for d in data]), dtype=torch.float64, device="cuda")
           for k in range(4)]
    total = sum(ns)
    m = torch.full((total,), W.M_DUST, dtype=torch.float64, device="cuda")
    kappa = torch.tensor([5e3, 6e3, 4.5e3], dtype=torch.float64, device="cuda")
    kc = torch.tensor([1e4, 2e4, 5e3], dtype=torch.float64, device="cuda")
    qc = torch.tensor([-1.6e-15, -1.2e-15, -2.0e-15], dtype=torch.float64, device="cuda")
    K = AdjointKernels(ns, gamma=3.0)
    K32 = AdjointKernels(ns, gamma=3.0, precision="fp32c")
    return K, ns, cat, m, kappa, kc, qc, K32


# relative-error bounds: FP64, and FP32 pair terms with Kahan sums
TOL = {"fp64": {"f": 1e-12, "pos": 1e-11, "vel": 1e-12, "q": 1e-11, "kappa": 1e-11, "kc": 1e-12},
       "fp32c": {"f": 1e-6, "pos": 1e-5, "vel": 1e-12, "q": 1e-5, "kappa": 1e-5, "kc": 1e-12}}


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_forces_match_dense_reference(setup, prec):
    K64, ns, (x, y, vx, vy), m, kappa, kc, qc, K32 = setup
    K = K64 if prec == "fp64" else K32
    K.set_params(kappa.cpu().numpy(), kc.cpu().numpy())
    q = qc[K.seg].contiguous()
    fx, fy, px, py = K.forces(x, y, vx, vy, q, m, pair=True)
    rx, ry = torch_forces(x, y, vx, vy, q, m, kappa, kc, 3.0, ns)
    err = torch.sqrt(((fx - rx) ** 2 + (fy - ry) ** 2).sum() / (rx**2 + ry**2).sum()).item()
    assert err < TOL[prec]["f"]
    zero = torch.zeros_like(kc)
    rpx, rpy = torch_forces(x, y, torch.zeros_like(vx), torch.zeros_like(vy), q, m, kappa, zero, 0.0, ns)
    err = torch.sqrt(((px - rpx) ** 2 + (py - rpy) ** 2).sum() / (rpx**2 + rpy**2).sum()).item()
    assert err < TOL[prec]["f"]


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_vjp_matches_torch_autograd(setup, prec):
    K64, ns, (x, y, vx, vy), m, kappa, kc, qc, K32 = setup
    K = K64 if prec == "fp64" else K32
    tol = TOL[prec]
    K.set_params(kappa.cpu().numpy(), kc.cpu().numpy())
    g = torch.Generator(device="cuda").manual_seed(3)
    ax = torch.randn(x.shape, dtype=torch.float64, device="cuda", generator=g)
    ay = torch.randn(x.shape, dtype=torch.float64, device="cuda", generator=g)
    q = qc[K.seg].contiguous()
    gx, gy, gvx, gvy, gq, gk, gc = K.vjp(x, y, vx, vy, q, m, ax, ay)
    leaves = [t.clone().requires_grad_(True) for t in (x, y, vx, vy, q)]
    kap = kappa.clone().requires_grad_(True)
    kcc = kc.clone().requires_grad_(True)
    rx, ry = torch_forces(*leaves[:4], leaves[4], m, kap, kcc, 3.0, ns)
    L = (ax * rx + ay * ry).sum()
    L.backward()

    def rel(a, b):
        return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()

    assert rel(gx, leaves[0].grad) < tol["pos"]
    assert rel(gy, leaves[1].grad) < tol["pos"]
    assert rel(gvx, leaves[2].grad) < tol["vel"]
    assert rel(gvy, leaves[3].grad) < tol["vel"]
    assert rel(gq, leaves[4].grad) < tol["q"]
    assert rel(K.per_cloud(gk), kap.grad) < tol["kappa"]
    assert rel(K.per_cloud(gc), kcc.grad) < tol["kc"]


def _loss(K, x0, y0, vx0, vy0, kappa, qc, kc, m, xt, yt, steps, every):
    from demon_simulation_code_gb300.adjoint import rollout

    xT, yT, _, _ = rollout(K, x0, y0, vx0, vy0, kappa, qc, kc, m, 1e-5, steps, every)
    return ((xT - xt) ** 2 + (yT - yt) ** 2).mean()


def test_rollout_gradient_vs_finite_differences_and_torch(setup):
    K, ns, (x, y, vx, vy), m, kappa, kc, qc, _ = setup
    steps, every = 23, 7  # a partial last segment
    xt = x + 1e-5
    yt = y - 2e-5
    x0 = x.clone().requires_grad_(True)
    kap = kappa.clone().requires_grad_(True)
    qq = qc.clone().requires_grad_(True)
    kcc = kc.clone().requires_grad_(True)
    L = _loss(K, x0, y, vx, vy, kap, qq, kcc, m, xt, yt, steps, every)
    L.backward()
    grads = {"kappa": kap.grad, "q": qq.grad, "kc": kcc.grad}

    def L_of(**over):
        args = dict(kappa=kappa, q=qc, kc=kc, x0=x)
        args.update(over)
        with torch.no_grad():
            return _loss(K, args["x0"], y, vx, vy, args["kappa"], args["q"], args["kc"], m, xt, yt,
                         steps, every).item()

    for name, base in (("kappa", kappa), ("q", qc), ("kc", kc)):
        for c in range(len(ns)):
            h = 1e-6 * abs(base[c].item())
            up = base.clone()
            dn = base.clone()
            up[c] += h
            dn[c] -= h
            fd = (L_of(**{name: up}) - L_of(**{name: dn})) / (2 * h)
            ad = grads[name][c].item()
            assert abs(ad - fd) <= 1e-4 * max(abs(fd), 1e-300), (name, c, ad, fd)
    for i in (0, 40, 105):
        h = 1e-6 * 6e-4
        up = x.clone()
        dn = x.clone()
        up[i] += h
        dn[i] -= h
        fd = (L_of(x0=up) - L_of(x0=dn)) / (2 * h)
        assert abs(x0.grad[i].item() - fd) <= 1e-4 * abs(fd) + 1e-12 * abs(L.item()) / 6e-4, (i,)

    # FP64 torch autograd through the same rollout (dense forces)
    def f(s, q, kapv, kcv):
        fx, fy = torch_forces(s[0], s[1], s[2], s[3], q, m, kapv, kcv, 3.0, ns)
        return (s[2], s[3], fx / m, fy / m)

    x0r = x.clone().requires_grad_(True)
    kapr = kappa.clone().requires_grad_(True)
    qr = qc.clone().requires_grad_(True)
    kcr = kc.clone().requires_grad_(True)
    qp = qr[K.seg]
    s = (x0r, y, vx, vy)
    dt = 1e-5
    for _ in range(steps):
        k1 = [dt * v for v in f(s, qp, kapr, kcr)]
        s2 = [a + 0.5 * b for a, b in zip(s, k1)]
        k2 = [dt * v for v in f(s2, qp, kapr, kcr)]
        s3 = [a + 0.5 * b for a, b in zip(s, k2)]
        k3 = [dt * v for v in f(s3, qp, kapr, kcr)]
        s4 = [a + b for a, b in zip(s, k3)]
        k4 = [dt * v for v in f(s4, qp, kapr, kcr)]
        s = tuple(a + (p + ((u + v) * 2.0 + w)) / 6.0 for a, p, u, v, w in zip(s, k1, k2, k3, k4))
    Lr = ((s[0] - xt) ** 2 + (s[1] - yt) ** 2).mean()
    Lr.backward()
    assert abs(Lr.item() - L.item()) <= 1e-12 * abs(L.item())
    for a, b in ((kap.grad, kapr.grad), (qq.grad, qr.grad), (kcc.grad, kcr.grad), (x0.grad, x0r.grad)):
        assert (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item() < 1e-9


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_kept_stage_inputs_give_the_checkpointed_gradients(setup, prec):
    """The backward pass from stage inputs kept by the forward pass and the
    one that recomputes them from checkpoints give the same bits."""
    from demon_simulation_code_gb300.adjoint import rollout

    K64, ns, (x, y, vx, vy), m, kappa, kc, qc, K32 = setup
    K = K64 if prec == "fp64" else K32
    out = []
    for keep in (True, False):
        leaves = [t.clone().requires_grad_(True) for t in (x, vy, kappa, qc, kc)]
        xT, yT, vxT, _ = rollout(K, leaves[0], y, vx, leaves[1], leaves[2], leaves[3], leaves[4], m, 1e-5,
                                 23, 7, keep_stages=keep)
        assert K.kept_stages is keep
        L = ((xT - x - 1e-5) ** 2 + (yT - y) ** 2).mean() + 1e-3 * (vxT ** 2).mean()
        L.backward()
        out.append([t.grad.clone() for t in leaves] + [L.detach()])
    for a, b in zip(*out):
        assert torch.equal(a, b)


class _AdjointOnTrajectory(AdjointKernels):
    """Forward steps (and the backward pass's recomputed steps) in one
    precision, the step adjoints in another: separates the adjoint's own
    error from that of the trajectory it is evaluated on."""

    def __init__(self, ns, forward, adjoint, **kw):
        super().__init__(ns, precision=forward, **kw)
        self._fwd = {"fp64": 0, "fp32c": 1}[forward]
        self._adj = {"fp64": 0, "fp32c": 1}[adjoint]

    def rk4_step(self, *a, **kw):
        self.precision = self._fwd
        return super().rk4_step(*a, **kw)

    def rk4_step_vjp(self, *a, **kw):
        self.precision = self._adj
        return super().rk4_step_vjp(*a, **kw)


def test_adjoint64_smooth_gradients_vs_finite_differences_and_fp64():
    """The 64 x 2048-particle, 200-step workload's shape on its first four
    clouds (clouds are independent, so each cloud's gradient is the same in
    the 64-cloud problem): FP32C and FP64 adjoint gradients of the loss with
    respect to kappa, q, k_c and initial positions against central finite
    differences (relative step 1e-6, FP64 rollouts), and FP32C against the
    FP64 adjoint gradient."""
    from demon_simulation_code_gb300.fit import TrajectoryFit

    w = W.adjoint64_smooth()
    sub = W.Workload(w.name, w.clouds[:4], w.dt, w.steps, extra=w.extra)
    f64 = TrajectoryFit(sub, precision="fp64")
    f32 = TrajectoryFit(sub, precision="fp32c")
    L64, g64 = f64.loss_and_grad()
    L32, g32 = f32.loss_and_grad()
    assert abs(L32.item() / L64.item() - 1) < 1e-6
    # FP64: every component to 1e-6 of itself.  FP32C: every component to
    # 1e-4 of the gradient's size (its largest component over the clouds); a
    # component far below that size carries FP32 rounding of the larger ones.
    for name in ("kappa", "q", "kc"):
        fd = f64.finite_difference(name)
        scale = fd.abs().max()
        print(name, "fd", fd.tolist(), "fp64", g64[name].tolist(), "fp32c", g32[name].tolist())
        assert ((g64[name] - fd).abs() / fd.abs()).max().item() < 1e-6, name
        assert ((g32[name] - fd).abs() / scale).max().item() < 1e-4, name
        assert ((g32[name] - g64[name]).abs() / scale).max().item() < 1e-4, name
    fd, idx = f64.finite_difference("x0", particles=[3, 510, 1029, 2047])
    scale = g64["x0"].abs().max()
    print("x0 fd", fd.tolist(), "fp64", g64["x0"][idx].tolist(), "fp32c", g32["x0"][idx].tolist())
    assert ((g64["x0"][idx] - fd).abs() / fd.abs()).max().item() < 1e-4
    assert ((g32["x0"][idx] - fd).abs() / scale).max().item() < 1e-4
    # over all 8192 initial positions, norm-wise.  On the same (FP64)
    # trajectory the FP32C step adjoint meets 1e-4 with room (measured
    # 2.7e-7); the FP32C gradient differs from the FP64 one by what its own
    # FP32C trajectory does to the loss (measured 5.1e-4; an FP64 adjoint on
    # the FP32C trajectory differs by the same), so that gate is looser.
    rel = ((g32["x0"] - g64["x0"]).norm() / g64["x0"].norm()).item()
    print("x0 fp32c vs fp64 norm-wise", rel)
    assert rel < 2e-3
    mixed = TrajectoryFit(sub, precision="fp64")
    mixed.K = _AdjointOnTrajectory(mixed.ns, flags=sub.clouds[0].flags, gamma=sub.clouds[0].gamma,
                                   forward="fp64", adjoint="fp32c")
    _, gm = mixed.loss_and_grad()
    rel_same = ((gm["x0"] - g64["x0"]).norm() / g64["x0"].norm()).item()
    print("x0 fp32c step adjoint on the fp64 trajectory vs fp64 norm-wise", rel_same)
    assert rel_same < 1e-5
    for name in ("kappa", "q", "kc"):
        assert ((gm[name] - g64[name]).abs() / g64[name].abs().max()).max().item() < 1e-5, name
