"""Learned warm start for the batched Jacobi solve.

The reference starts every substep's Jacobi solve from the predicted positions
(``XPBD.py:116-118``) and has no learned part.  Here a per-vertex MLP
(24 -> 64 -> 64 -> 3, SiLU, BF16 weights and activations, FP32 accumulation on
tensor cores; ``csrc/sx_learned.cu``) predicts the correction the solve will
make, in units of the vertex's mean spring rest length, from local features of
the predicted state: the spring and bending correction directions, strains,
the predicted displacement, the previous substep's correction, the pin flag,
the vertex degree and gravity.  The solve then starts from
``y_pred + fixed * L * correction``; if that start has a larger constraint
residual than ``y_pred`` itself, the solver falls back to the cold start (a
device-side decision, inside the captured graph).

Training data are generated by the plain solver: :class:`WarmStart` in
``"record"`` mode computes the features after each prediction and, after the
solve, the target ``(y_final - y_pred) / L``.  :class:`WarmStartMLP` trains on
them with the library's own forward/backward kernels and Adam.
"""
from __future__ import annotations

import numpy as np
import torch

from ._lib import ptr, stream_handle, sx

SHAPES = [("W1", (64, 32)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (8, 64)), ("b3", (8,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)
N_BF16 = 64 * 32 + 64 * 64 + 8 * 64
N_FEATURES = 24


def init_params(seed: int = 0) -> np.ndarray:
    """Uniform fan-in initialisation; the output layer starts small so that an
    untrained network predicts almost no correction.  Structurally zero
    entries (W1 columns >= 24, W3 rows >= 3, b3[3:]) are zero."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in SHAPES:
        if name.startswith("b"):
            a = np.zeros(shape, np.float32)
        else:
            fan_in = N_FEATURES if name == "W1" else shape[1]
            lim = np.sqrt(3.0 / fan_in) * (0.1 if name == "W3" else 1.0)
            a = rng.uniform(-lim, lim, shape).astype(np.float32)
            if name == "W1":
                a[:, N_FEATURES:] = 0
            if name == "W3":
                a[3:] = 0
        parts.append(a.ravel())
    return np.concatenate(parts).astype(np.float32)


def zero_output_params(seed: int = 0) -> np.ndarray:
    """init_params with the output layer zeroed: a network that predicts no
    correction, whose evaluate_loss is the loss of the cold start under the
    same masked loss function."""
    p = init_params(seed)
    o = 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        if name in ("W3", "b3"):
            p[o:o + n] = 0.0
        o += n
    return p


def mean_spring_rest(adj_ptr: np.ndarray, adj: np.ndarray) -> np.ndarray:
    """L per vertex: mean rest length of its springs (of all its constraints if
    it has none, 1 if it has no constraint)."""
    V = adj_ptr.shape[0] - 1
    owner = np.repeat(np.arange(V), np.diff(adj_ptr))
    rest = adj[:, 1].view(np.float32).astype(np.float64)
    spring = adj[:, 0] >= 0
    ss = np.bincount(owner[spring], weights=rest[spring], minlength=V)
    sn = np.bincount(owner[spring], minlength=V)
    aa = np.bincount(owner, weights=rest, minlength=V)
    an = np.bincount(owner, minlength=V)
    L = np.where(sn > 0, ss / np.maximum(sn, 1), np.where(an > 0, aa / np.maximum(an, 1), 1.0))
    return L.astype(np.float32)


class WarmStartMLP:
    """Parameters, Adam state and the library calls of the warm-start MLP.

    Inference runs on the tcgen05 tensor cores (``sx_mlp_forward_tc``: 128-row
    tiles, accumulators in tensor memory) unless ``tcgen05`` is False, which
    selects the mma.sync kernel (``sx_mlp_forward``) that training's forward
    pass shares; the two agree to the BF16 rounding of the hidden activations.
    """

    def __init__(self, device="cuda", seed: int = 0, params: np.ndarray | None = None, tcgen05: bool = True):
        if int(sx.sx_mlp_param_count()) != N_PARAMS or int(sx.sx_mlp_bf16_count()) != N_BF16:
            raise RuntimeError("MLP layout of the library does not match")
        self.device = torch.device(device)
        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        self.p32 = torch.from_numpy(p.copy()).to(self.device)
        self.w16 = torch.zeros(N_BF16, dtype=torch.bfloat16, device=self.device)
        self.adam_m = torch.zeros_like(self.p32)
        self.adam_v = torch.zeros_like(self.p32)
        self.grad = torch.zeros_like(self.p32)
        self.stats = torch.zeros(4, dtype=torch.float32, device=self.device)
        self.step = 0
        self._ws = None
        self._ws_rows = 0
        self.tcgen05 = tcgen05
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)  # SX_STATUS_* of the tcgen05 path
        self.sync()

    def sync(self):
        sx.sx_mlp_sync_bf16(ptr(self.p32), ptr(self.w16), stream_handle())

    def forward(self, feat: torch.Tensor, out4: torch.Tensor, n_rows: int | None = None):
        n = feat.shape[0] if n_rows is None else n_rows
        if self.tcgen05:
            sx.sx_mlp_forward_tc(ptr(feat), n, ptr(self.w16), ptr(self.p32), ptr(out4), ptr(self.status),
                                 stream_handle())
        else:
            sx.sx_mlp_forward(ptr(feat), n, ptr(self.w16), ptr(self.p32), ptr(out4), stream_handle())
        return out4

    def _workspace(self, rows: int):
        if self._ws is None or self._ws_rows < rows:
            nbytes = int(sx.sx_mlp_train_workspace_bytes(rows))
            self._ws = torch.zeros(nbytes, dtype=torch.uint8, device=self.device)
            self._ws_rows = rows
        return self._ws

    def gradients(self, feat, target4, idx, n_valid: int):
        """Gradient of the masked MSE over rows idx (device tensor) and n_valid*loss."""
        ws = self._workspace(idx.shape[0])
        sx.sx_mlp_gradients(ptr(feat), ptr(target4), ptr(idx), idx.shape[0], int(n_valid), ptr(self.w16),
                            ptr(self.p32), ptr(self.grad), ptr(self.stats), ptr(ws), ws.numel(), stream_handle())
        return self.grad, self.stats

    def train_step(self, feat, target4, idx, n_valid: int, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        """One Adam step; returns the device stats tensor (stats[0] = n_valid * loss)."""
        ws = self._workspace(idx.shape[0])
        self.step += 1
        sx.sx_mlp_train_step(ptr(feat), ptr(target4), ptr(idx), idx.shape[0], int(n_valid), ptr(self.w16),
                             ptr(self.p32), ptr(self.adam_m), ptr(self.adam_v), float(lr), float(betas[0]),
                             float(betas[1]), float(eps), self.step, ptr(self.stats), ptr(ws), ws.numel(),
                             stream_handle())
        return self.stats

    def params(self) -> np.ndarray:
        return self.p32.detach().cpu().numpy().copy()

    def save(self, path):
        np.savez(path, params=self.params())

    @classmethod
    def load(cls, path, device="cuda"):
        with np.load(path) as z:
            return cls(device=device, params=z["params"])


class WarmStart:
    """Warm-start plumbing for a :class:`BatchedSolver` (``solver.warm = ...``).

    ``mode="apply"``: predict a start with the MLP and keep it unless it raises
    the residual.  ``mode="record"``: leave the cold start alone and record
    features and targets for training (``feat``, ``target4`` after each
    substep; ``on_substep`` is called with them)."""

    def __init__(self, solver, mlp: WarmStartMLP | None = None, mode: str = "apply"):
        if mode not in ("apply", "record"):
            raise ValueError("mode must be 'apply' or 'record'")
        if mode == "apply" and mlp is None:
            raise ValueError("apply mode needs a network")
        self.mode = mode
        self.mlp = mlp
        dev = solver.device
        V = solver.num_verts
        self.V = V
        self.Lref = torch.from_numpy(
            mean_spring_rest(solver.adj_ptr.cpu().numpy(), solver.adj.cpu().numpy())).to(dev)
        self.y_pred = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self.c4 = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self.feat = torch.zeros((V, 32), dtype=torch.bfloat16, device=dev)
        self.out4 = torch.zeros((V, 4), dtype=torch.float32, device=dev)
        self.target4 = torch.zeros((V, 4), dtype=torch.float32, device=dev) if mode == "record" else None
        self.res_cold = torch.zeros(4, dtype=torch.float64, device=dev)
        self.res_warm = torch.zeros(4, dtype=torch.float64, device=dev)
        self.flags = torch.zeros(2, dtype=torch.int32, device=dev)
        self._ws = torch.zeros(int(sx.sx_residual_workspace_bytes(V)), dtype=torch.uint8, device=dev)
        self.on_substep = None

    def reset(self):
        self.c4.zero_()
        self.flags.zero_()

    def begin(self, solver, dt: float):
        """After the prediction: features, and in apply mode the warm start."""
        s = stream_handle()
        g = solver.g
        sx.sx_warm_features(ptr(solver.x4), ptr(solver.y4), ptr(self.c4), ptr(solver.fixed), ptr(solver.adj_ptr),
                            ptr(solver.adj), ptr(self.Lref), self.V, g[0], g[1], g[2], float(dt), ptr(self.feat),
                            ptr(self.y_pred), s)
        if self.mode != "apply":
            return
        self.mlp.forward(self.feat, self.out4)
        sx.sx_constraint_residual(ptr(solver.y4), ptr(solver.adj_ptr), ptr(solver.adj), self.V, ptr(self.res_cold),
                                  ptr(self._ws), self._ws.numel(), s)
        sx.sx_warm_apply(ptr(self.y_pred), ptr(self.out4), ptr(solver.fixed), ptr(self.Lref), self.V,
                         ptr(solver.y4), s)
        sx.sx_constraint_residual(ptr(solver.y4), ptr(solver.adj_ptr), ptr(solver.adj), self.V, ptr(self.res_warm),
                                  ptr(self._ws), self._ws.numel(), s)
        sx.sx_warm_select(ptr(self.res_warm), ptr(self.res_cold), ptr(self.y_pred), ptr(solver.y4), self.V,
                          ptr(self.flags), s)

    def end(self, solver):
        """After the solve: the correction for the next substep's features (and
        the training target in record mode)."""
        sx.sx_warm_record(ptr(solver.y4), ptr(self.y_pred), ptr(solver.fixed), ptr(self.Lref), self.V, ptr(self.c4),
                          ptr(self.target4) if self.target4 is not None else None, stream_handle())
        if self.on_substep is not None:
            self.on_substep(self)

    def fallback_counts(self):
        f = self.flags.cpu().tolist()
        return {"cold_fallbacks": f[0], "warm_starts": f[1]}


def collect_samples(solver, frames: int, rows_per_substep: int, n_substeps: int = 10, seed: int = 0):
    """Run the plain solver for ``frames`` frames with a recording WarmStart and
    keep ``rows_per_substep`` random free vertices of every substep.
    Returns (feat[N, 32] bf16, target4[N, 4]) on the solver's device."""
    ws = WarmStart(solver, mode="record")
    gen = torch.Generator(device=solver.device)
    gen.manual_seed(seed)
    free = torch.nonzero(solver.fixed > 0).flatten()
    feats, targets = [], []

    def grab(w):
        pick = free[torch.randint(free.numel(), (rows_per_substep,), device=solver.device, generator=gen)]
        feats.append(w.feat.index_select(0, pick))
        targets.append(w.target4.index_select(0, pick))

    ws.on_substep = grab
    prev_warm, prev_graph = solver.warm, solver.use_graph
    solver.warm, solver.use_graph = ws, False
    try:
        for _ in range(frames):
            solver.forward(n_substeps)
    finally:
        solver.warm, solver.use_graph = prev_warm, prev_graph
    return torch.cat(feats), torch.cat(targets)


def train(mlp: WarmStartMLP, feat, target4, steps: int, batch: int = 65536, lr: float = 2e-3, seed: int = 0,
          log_every: int = 0):
    """Adam on random minibatches; returns the per-step losses (host floats,
    read back every ``log_every`` steps, or only at the end)."""
    gen = torch.Generator(device=feat.device)
    gen.manual_seed(seed)
    N = feat.shape[0]
    losses = []
    hist = torch.zeros(steps, dtype=torch.float32, device=feat.device)
    for k in range(steps):
        idx = torch.randint(N, (batch,), device=feat.device, generator=gen, dtype=torch.int32)
        n_valid = batch  # every sampled row is a free vertex
        st = mlp.train_step(feat, target4, idx, n_valid, lr=lr)
        hist[k] = st[0] / n_valid
        if log_every and (k + 1) % log_every == 0:
            losses.append(float(hist[k].item()))
    return hist.cpu().numpy()


def evaluate_loss(mlp: WarmStartMLP, feat, target4, rows: int | None = None) -> float:
    """Mean masked loss over the first ``rows`` samples (all by default)."""
    n = feat.shape[0] if rows is None else min(rows, feat.shape[0])
    idx = torch.arange(n, dtype=torch.int32, device=feat.device)
    n_valid = int((target4[:n, 3] > 0).sum().item())
    _, st = mlp.gradients(feat, target4, idx, max(n_valid, 1))
    return float(st[0].item()) / max(n_valid, 1)
