"""Learned warm start: the oracle's MLP gradients against finite differences,
the features restated literally, and (GPU) the CUDA features, forward pass and
gradients against the oracle."""
import numpy as np
import pytest
import torch


def _random_batch(po, rng, n=64):
    feat = po.bf16_round(rng.normal(0, 1, (n, 32)).astype(np.float32))
    feat[:, 24:] = 0
    u16 = (feat.view(np.uint32) >> 16).astype(np.uint16)
    t = np.zeros((n, 4), np.float32)
    t[:, :3] = rng.normal(0, 0.5, (n, 3))
    t[:, 3] = (rng.uniform(size=n) > 0.2).astype(np.float32)
    return u16, t


def _params(pkg, seed=0, out_scale=3.0):
    p = pkg.learned.init_params(seed)
    o = 64 * 32 + 64 + 64 * 64 + 64
    p[o:o + 3 * 64] *= out_scale  # a non-trivial output layer
    return p


def test_mlp_backward_formulas_finite_difference(pkg, po):
    rng = np.random.default_rng(0)
    u16, t = _random_batch(po, rng, 32)
    p = _params(pkg).astype(np.float64)
    g = po.mlp_gradients64(u16, t, p)
    h = 1e-6
    for i in rng.choice(np.flatnonzero(np.abs(g) > 1e-6), 40, replace=False):
        e = np.zeros_like(p)
        e[i] = h
        fd = (po.mlp_loss64(u16, t, p + e) - po.mlp_loss64(u16, t, p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])


def test_mlp_rounded_gradients_near_exact(pkg, po):
    """The BF16-rounded gradient the kernels compute stays close to the exact one."""
    rng = np.random.default_rng(1)
    u16, t = _random_batch(po, rng, 256)
    p = _params(pkg, seed=1)
    g32, loss, n_valid = po.mlp_gradients(u16, t, p)
    g64 = po.mlp_gradients64(u16, t, p.astype(np.float64))
    assert np.linalg.norm(g32 - g64) <= 0.03 * np.linalg.norm(g64)
    assert abs(loss / n_valid - po.mlp_loss64(u16, t, p)) <= 0.02 * loss / n_valid


def _features_literal(po, x4, y4, c4, fixed, ptr, adj, L, g, dt):
    """Plain-Python float32 restatement of the feature definition."""
    f32 = np.float32
    V = y4.shape[0]
    out = np.zeros((V, 32), np.float32)
    for v in range(V):
        ps, xs, cp = y4[v], x4[v], c4[v]
        inv = f32(1) / f32(L[v])
        S = [f32(0)] * 3
        Bv = [f32(0)] * 3
        sa = ba = smax = smin = f32(0)
        ns = nb = 0
        for k in range(ptr[v], ptr[v + 1]):
            w = int(adj[k, 0])
            rest = adj[k, 1:2].view(np.float32)[0]
            o = y4[w & 0x7FFFFFFF]
            e = [f32(ps[i] - o[i]) for i in range(3)]
            ln = f32(np.sqrt(f32(f32(e[0] * e[0] + e[1] * e[1]) + e[2] * e[2])))
            C = f32(ln - rest)
            il = f32(1) / ln if ln > 0 else f32(0)
            c = [f32(C * f32(il * e[i])) for i in range(3)]
            r = f32(C / rest) if rest > 0 else f32(0)
            if w < 0:
                Bv = [f32(Bv[i] + c[i]) for i in range(3)]
                ba = f32(ba + abs(r))
                nb += 1
            else:
                S = [f32(S[i] + c[i]) for i in range(3)]
                sa = f32(sa + abs(r))
                smax = max(smax, r) if ns else r
                smin = min(smin, r) if ns else r
                ns += 1
        fs, fb = f32(ns), f32(nb)
        d = [f32(ps[i] - xs[i]) for i in range(3)]
        f = [(-f32(f32(S[i] / fs) * inv) if ns else f32(0)) for i in range(3)]
        f += [(-f32(f32(Bv[i] / fb) * inv) if nb else f32(0)) for i in range(3)]
        f += [f32(sa / fs) if ns else f32(0), smax, smin, f32(ba / fb) if nb else f32(0)]
        f += [f32(d[i] * inv) for i in range(3)] + [f32(cp[i] * inv) for i in range(3)]
        f += [f32(fixed[v]), f32(fs / f32(6)), f32(fb / f32(6))]
        f += [f32(f32(np.sqrt(f32(f32(cp[0] * cp[0] + cp[1] * cp[1]) + cp[2] * cp[2]))) * inv)]
        f += [f32(f32(np.sqrt(f32(f32(d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]))) * inv)]
        f += [f32(f32(f32(g[i]) * f32(dt)) * f32(dt)) * inv for i in range(3)]
        out[v, :24] = [min(max(x, f32(-16)), f32(16)) for x in f]
    return out


def _feature_inputs(pkg, po, n=7, seed=0):
    rng = np.random.default_rng(seed)
    x, f = pkg.grid_cloth(n)
    e = pkg.mesh.edges_from_faces(f)
    b = pkg.mesh.bending_pairs(f)
    l0 = pkg.mesh.rest_lengths(x, e)
    bl0 = pkg.mesh.rest_lengths(x, b)
    ptr, adj = po.adjacency(x.shape[0], e, l0, b, bl0)
    V = x.shape[0]
    x4 = np.zeros((V, 4), np.float32)
    x4[:, :3] = x
    y4 = x4.copy()
    y4[:, :3] += rng.normal(0, 2e-3, (V, 3)).astype(np.float32)
    c4 = np.zeros((V, 4), np.float32)
    c4[:, :3] = rng.normal(0, 1e-3, (V, 3))
    fixed = np.ones(V, np.float32)
    fixed[[0, n - 1]] = 0
    L = pkg.learned.mean_spring_rest(ptr, adj)
    return x4, y4, c4, fixed, ptr, adj, L


def test_warm_features_literal(pkg, po):
    x4, y4, c4, fixed, ptr, adj, L = _feature_inputs(pkg, po)
    g, dt = (0.0, 0.0, -9.81), 1 / 600
    feat = po.warm_features(x4, y4, c4, fixed, ptr, adj, L, g, dt)
    lit = _features_literal(po, x4, y4, c4, fixed, ptr, adj, L, g, dt)
    assert np.array_equal(po.bf16_to_f32(feat), po.bf16_round(lit))


def test_init_params_layout(pkg, po):
    p = pkg.learned.init_params(3)
    assert p.shape == (po.MLP_PARAMS,) == (pkg.learned.N_PARAMS,)
    P = po.mlp_unpack(p)
    assert not P["W1"][:, 24:].any() and not P["W3"][3:].any() and not P["b3"].any()


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_warm_features_bit_exact(pkg, po):
    x4, y4, c4, fixed, ptr, adj, L = _feature_inputs(pkg, po, n=40, seed=2)
    from starlab_physics_gb300._lib import ptr as dptr, stream_handle, sx

    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    V = x4.shape[0]
    feat = torch.zeros((V, 32), dtype=torch.bfloat16, device="cuda")
    yp = torch.zeros((V, 4), dtype=torch.float32, device="cuda")
    # every device array stays referenced until the kernel has finished
    dx4, dy4, dc4, dfix, dptr_, dadj, dL = (t(a) for a in (x4, y4, c4, fixed, ptr, adj, L))
    sx.sx_warm_features(dptr(dx4), dptr(dy4), dptr(dc4), dptr(dfix), dptr(dptr_), dptr(dadj), dptr(dL), V, 0.0, 0.0,
                        -9.81, 1 / 600, dptr(feat), dptr(yp), stream_handle())
    torch.cuda.synchronize()
    got = feat.view(torch.int16).cpu().numpy().view(np.uint16)
    ref = po.warm_features(x4, y4, c4, fixed, ptr, adj, L, (0.0, 0.0, -9.81), 1 / 600)
    assert np.array_equal(got, ref)
    assert torch.equal(yp, dy4)


def _gpu_batch(po, rng, n):
    u16, t = _random_batch(po, rng, n)
    feat = torch.from_numpy(u16.view(np.int16)).cuda().view(torch.bfloat16)
    return u16, t, feat, torch.from_numpy(t).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [16, 1000, 70001])
def test_mlp_forward_matches_oracle(pkg, po, n):
    """The mma.sync forward (shared with training) against the oracle."""
    rng = np.random.default_rng(n)
    u16, _, feat, _ = _gpu_batch(po, rng, n)
    p = _params(pkg, seed=n % 7)
    mlp = pkg.WarmStartMLP(params=p, tcgen05=False)
    out = torch.full((n, 4), np.nan, dtype=torch.float32, device="cuda")
    mlp.forward(feat, out)
    got = out.cpu().numpy()
    ref = po.mlp_forward(u16, p)
    scale = np.abs(ref[:, :3]).max()
    assert np.abs(got[:, :3] - ref[:, :3]).max() <= 1e-2 * scale
    assert np.abs(got[:, :3] - ref[:, :3]).mean() <= 1e-3 * scale
    assert not got[:, 3].any()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [16, 129, 1000, 70001])
def test_mlp_forward_tcgen05_matches(pkg, po, n):
    """The tcgen05 forward (128-row tiles, accumulators in tensor memory)
    against the oracle (same tolerance as the mma.sync forward) and against the
    mma.sync forward (FP32 accumulation order and the bias step differ; the
    BF16 hidden activations may round differently by one unit)."""
    from starlab_physics_gb300._lib import ptr, stream_handle, sx

    rng = np.random.default_rng(n + 1)
    u16, _, feat, _ = _gpu_batch(po, rng, n)
    p = _params(pkg, seed=n % 5)
    mlp = pkg.WarmStartMLP(params=p, tcgen05=False)
    ref_gpu = torch.full((n, 4), np.nan, dtype=torch.float32, device="cuda")
    mlp.forward(feat, ref_gpu)
    out = torch.full((n, 4), np.nan, dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert sx.sx_mlp_forward_tc(ptr(feat), n, ptr(mlp.w16), ptr(mlp.p32), ptr(out), ptr(status), stream_handle()) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got = out.cpu().numpy()
    ref = po.mlp_forward(u16, p)
    scale = np.abs(ref[:, :3]).max()
    assert np.isfinite(got).all()
    assert np.abs(got[:, :3] - ref[:, :3]).max() <= 1e-2 * scale
    assert np.abs(got[:, :3] - ref[:, :3]).mean() <= 1e-3 * scale
    assert not got[:, 3].any()
    g2 = ref_gpu.cpu().numpy()
    assert np.abs(got[:, :3] - g2[:, :3]).max() <= 1e-2 * scale


@pytest.mark.gpu
@pytest.mark.parametrize("n", [48, 5000, 70001])
def test_mlp_gradients_match_oracle(pkg, po, n):
    """Gradients and loss against the oracle; the partial sums are added in a
    fixed order, so a repeated call gives the same bits."""
    rng = np.random.default_rng(10 + n)
    u16, t, feat, tt = _gpu_batch(po, rng, n)
    p = _params(pkg, seed=2)
    mlp = pkg.WarmStartMLP(params=p)
    perm = rng.permutation(n).astype(np.int32)
    idx = torch.from_numpy(perm).cuda()
    n_valid = int(t[:, 3].sum())
    grad, st = mlp.gradients(feat, tt, idx, n_valid)
    g = grad.cpu().numpy().copy()
    loss_gpu = float(st[0].item())
    grad2, st2 = mlp.gradients(feat, tt, idx, n_valid)
    assert np.array_equal(grad2.cpu().numpy(), g) and float(st2[0].item()) == loss_gpu
    ref, loss, _ = po.mlp_gradients(u16[perm], t[perm], p)
    assert np.linalg.norm(g - ref) <= 2e-2 * np.linalg.norm(ref)
    assert abs(loss_gpu - loss) <= 1e-3 * loss
    # structurally zero entries stay zero
    P = po.mlp_unpack(g)
    assert not P["W1"][:, 24:].any() and not P["W3"][3:].any() and not P["b3"][3:].any()


@pytest.mark.gpu
def test_adam_step_matches_reference(pkg, po):
    """One train step = gradient + Adam (FP32) on the master weights."""
    rng = np.random.default_rng(7)
    u16, t, feat, tt = _gpu_batch(po, rng, 3000)
    p = _params(pkg, seed=4)
    mlp = pkg.WarmStartMLP(params=p)
    idx = torch.arange(3000, dtype=torch.int32, device="cuda")
    n_valid = int(t[:, 3].sum())
    grad, _ = mlp.gradients(feat, tt, idx, n_valid)
    g = grad.cpu().numpy().copy()
    mlp.train_step(feat, tt, idx, n_valid, lr=1e-3)
    got = mlp.params()
    m = 0.1 * g
    v = 0.001 * g * g
    ref = p - 1e-3 * ((m / 0.1) / (np.sqrt(v / 0.001) + 1e-8))
    P = po.mlp_unpack(ref)
    P["W1"][:, 24:] = 0
    P["W3"][3:] = 0
    P["b3"][3:] = 0
    ref = np.concatenate([P[k].ravel() for k, _ in po.MLP_SHAPES])
    assert np.allclose(got, ref, rtol=1e-5, atol=1e-7)


def _small_batch(pkg, seed, n_inst=96):
    insts = pkg.batched_scene(n_inst, seed=seed, n_min=16, n_max=64)
    return pkg.BatchedSolver(insts, dHat=(4e-3) ** 2, stiffness_stretch=1e5, stiffness_bending=1e8,
                             g=(0.0, 0.0, -9.81), dt=1.0 / 60.0, n_iter=20, padding=8e-3)


@pytest.fixture(scope="module")
def trained(pkg):
    """A network trained on samples of the plain solver (seed-0 scene, 80
    iterations per substep, frames 2-15: free fall and the first contacts
    with the boxes), with its loss history and held-out samples of another
    scene over the same frames."""
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = pkg.learned
    A = _small_batch(pkg, 0)
    A.forward(10)
    A.n_iter = 80
    feat, tgt = L.collect_samples(A, frames=14, rows_per_substep=8192)
    B = _small_batch(pkg, 1)
    B.forward(10)
    B.n_iter = 80
    vf, vt = L.collect_samples(B, frames=14, rows_per_substep=2048, seed=3)
    mlp = pkg.WarmStartMLP(seed=0)
    before = L.evaluate_loss(mlp, vf, vt)
    h1 = L.train(mlp, feat, tgt, 3000, batch=16384, lr=2e-3)
    h2 = L.train(mlp, feat, tgt, 1000, batch=16384, lr=5e-4)
    return mlp, np.concatenate([h1, h2]), before, vf, vt


@pytest.mark.gpu
def test_training_reduces_loss(pkg, trained):
    """Training on solver-generated samples lowers the loss on the training
    samples and on held-out samples from another scene, below the loss of
    predicting no correction."""
    L = pkg.learned
    mlp, hist, before, vf, vt = trained
    after = L.evaluate_loss(mlp, vf, vt)
    zero = L.evaluate_loss(pkg.WarmStartMLP(params=L.zero_output_params()), vf, vt)
    assert zero == pytest.approx(float(vt[:, :3].pow(2).sum(1).mean().item()), rel=1e-3)
    assert np.all(np.isfinite(hist))
    # the samples span free fall and contact, whose corrections the features
    # only partly determine: the loss falls severalfold, not to zero
    assert hist[-50:].mean() < 0.5 * hist[:10].mean(), (hist[-50:].mean(), hist[:10].mean())
    assert after < 0.3 * before, (after, before)
    assert after < 0.9 * zero, (after, zero)


@pytest.mark.gpu
def test_warm_start_gain(pkg, trained):
    """What the trained network gains: on a held-out scene, from the same
    substep starts, the warm-started solve with k Jacobi iterations ends closer
    to a converged solve (200 iterations) than the cold-started solve with the
    same k; and iterating to a residual tolerance relative to the cold start,
    the warm start stops earlier (device-side loop in a captured frame)."""
    L = pkg.learned
    mlp = trained[0]
    B = _small_batch(pkg, 1)
    rec = L.WarmStart(B, mode="record")
    B.warm = rec
    for _ in range(12):  # into the contact phase for the higher boxes
        B.forward(10)
    B.warm = None
    snap = (B.x4.clone(), B.v4.clone(), rec.c4.clone())
    dt = B.dt / 10
    warm = L.WarmStart(B, mlp)

    def run(n_iter, w=None):
        B.x4.copy_(snap[0])
        B.v4.copy_(snap[1])
        B.n_iter, B.warm = n_iter, w
        if w is not None:
            w.c4.copy_(snap[2])
        B.substep(dt)
        return B.x4[:, :3].clone()

    ref = run(200)
    for k in (4, 8):
        e_plain = float((run(k) - ref).norm(dim=1).pow(2).mean().sqrt())
        e_warm = float((run(k, warm) - ref).norm(dim=1).pow(2).mean().sqrt())
        assert e_warm < 0.9 * e_plain, (k, e_warm, e_plain)
    stops = {}
    for mode in ("plain", "learned"):
        B.x4.copy_(snap[0])
        B.v4.copy_(snap[1])
        B.tol, B.tol_relative, B.check_every, B.n_iter, B.use_graph = 0.995, True, 4, 200, True
        B.warm = L.WarmStart(B, mlp) if mode == "learned" else None
        if B.warm is not None:
            B.warm.c4.copy_(snap[2])
        B.convergence_stats(reset=True)
        B.forward(10)
        st = B.convergence_stats()
        assert st["converged_substeps"] == 10, (mode, st)
        stops[mode] = st["mean_stop_iteration"]
    B.warm = None
    assert stops["learned"] <= stops["plain"], stops
