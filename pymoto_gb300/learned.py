"""Learned warm start of the FP64 flexible CG: a small 3D convolutional network on the device.

The reference has no learned component: LinSolve starts every solve from the previous solution
(pymoto/modules/linalg.py:195) and its LDAWrapper projects the right-hand side on stored solution pairs
(pymoto/solvers/solvers.py:170-250).  Here a 3-level encoder-decoder (16/32/64 channels, 3x3x3 kernels,
BF16 weights and activations, FP32 accumulation) maps the element stiffness field of a design to the
displacement field on the nodes of a coarse multigrid level.  Its prediction, prolongated to the fine
grid, and the previous solution span a 2-dimensional space in which the initial guess is the
energy-optimal (Rayleigh-Ritz) combination, so the initial error in the K-norm is never larger than with
the previous solution alone; every solve is still driven to the same FP64 residual tolerance.

The network is trained on the device, online, on (stiffness field, displacement) pairs of the solves of
earlier design iterations (and optionally of seeded random density fields), by the forward and backward
kernels of libpymoto_gb300 (csrc/learned.cu: BF16 tensor-core convolutions) and an Adam update.  Targets are
normalised to unit 2-norm: the Rayleigh-Ritz step picks the scale.  The training steps run on a side stream
of their own, off the solver's critical path; the next prediction waits for them.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib
from ._lib import F32, F64, MATVEC, RESIDUAL, call, stream

# (name, cin, cout, relu)
LAYERS = [("enc1a", 4, 16, True), ("enc1b", 16, 16, True), ("enc2a", 16, 32, True), ("enc2b", 32, 32, True),
          ("enc3a", 32, 64, True), ("enc3b", 64, 64, True), ("dec2", 96, 32, True), ("dec1", 48, 16, True),
          ("head", 16, 3, False)]


def _nw(cin, cout):
    return 27 * cin * cout + cout


class ConvNet3D:
    """The encoder-decoder on a voxel grid (nx, ny, nz) (each divisible by 4), batch size 1.

    Parameters: one flat FP32 master array (per layer [w[tap][cin][cout], bias[cout]]) with its BF16 copy,
    gradient and Adam moments.  forward() reads `self.feat` (BF16 [v][4]) and writes `self.out` (FP32
    [v][3]); backward() takes dL/d(out) in `self.d_out` and writes the parameter gradient `self.grad`.
    """

    def __init__(self, vgrid, device="cuda", seed=0):
        nx, ny, nz = vgrid
        if nx % 4 or ny % 4 or nz % 4:
            raise ValueError("voxel grid must be divisible by 4 (two 2x poolings)")
        self.g1 = (nx, ny, nz)
        self.g2 = (nx // 2, ny // 2, nz // 2)
        self.g3 = (nx // 4, ny // 4, nz // 4)
        self.v1, self.v2, self.v3 = (int(np.prod(g)) for g in (self.g1, self.g2, self.g3))
        self.device = device
        self.offsets = {}
        off = 0
        for name, cin, cout, _ in LAYERS:
            self.offsets[name] = (off, cin, cout)
            off += _nw(cin, cout)
        self.nparam = off
        f32 = dict(dtype=torch.float32, device=device)
        bf = dict(dtype=torch.bfloat16, device=device)
        gen = torch.Generator().manual_seed(seed)
        w = torch.zeros(self.nparam, dtype=torch.float32)
        for name, cin, cout, relu in LAYERS:
            o = self.offsets[name][0]
            std = math.sqrt(2.0 / (27 * cin)) if relu else 0.1 * math.sqrt(1.0 / (27 * cin))
            w[o:o + 27 * cin * cout] = torch.randn(27 * cin * cout, generator=gen) * std
        self.w = w.to(device)
        self.w_bf = self.w.to(torch.bfloat16)
        self.grad = torch.zeros(self.nparam, **f32)
        self.m = torch.zeros(self.nparam, **f32)
        self.v = torch.zeros(self.nparam, **f32)
        self.step_count = 0
        v1, v2, v3 = self.v1, self.v2, self.v3
        # activations (BF16) and their gradients (FP32)
        A = lambda n, c: torch.zeros(n * c, **bf)   # noqa: E731
        G = lambda n, c: torch.zeros(n * c, **f32)  # noqa: E731
        self.feat = A(v1, 4)
        self.a1, self.a2, self.p2 = A(v1, 16), A(v1, 16), A(v2, 16)
        self.a3, self.a4, self.p3 = A(v2, 32), A(v2, 32), A(v3, 32)
        self.a5, self.a6 = A(v3, 64), A(v3, 64)
        self.cat2, self.a7 = A(v2, 96), A(v2, 32)
        self.cat1, self.a8 = A(v1, 48), A(v1, 16)
        self.out = G(v1, 3)
        self.d_out, self.d_a8, self.d_cat1, self.d_a2, self.d_a1 = G(v1, 3), G(v1, 16), G(v1, 48), G(v1, 16), G(v1, 16)
        self.d_a7, self.d_cat2, self.d_a4, self.d_a3, self.d_p2 = G(v2, 32), G(v2, 96), G(v2, 32), G(v2, 32), G(v2, 16)
        self.d_a6, self.d_a5, self.d_p3 = G(v3, 64), G(v3, 64), G(v3, 32)
        lib = _lib.load()
        nbytes = 0
        for grid, (_, cin, cout) in [(self.g1, self.offsets["enc1a"]), (self.g1, self.offsets["enc1b"]),
                                     (self.g2, self.offsets["enc2a"]), (self.g2, self.offsets["enc2b"]),
                                     (self.g3, self.offsets["enc3a"]), (self.g3, self.offsets["enc3b"]),
                                     (self.g2, self.offsets["dec2"]), (self.g1, self.offsets["dec1"]),
                                     (self.g1, self.offsets["head"])]:
            nbytes = max(nbytes, lib.pmg_nn_wgrad_scratch_bytes(*grid, cin, cout))
        self.scratch = torch.zeros(nbytes // 4 + 1, **f32)

    # parameter views -----------------------------------------------------------------------------
    def _w(self, name):
        o = self.offsets[name][0]
        return self.w_bf[o:]

    def _b(self, name):
        o, cin, cout = self.offsets[name]
        return self.w[o + 27 * cin * cout:]

    def _g(self, name):
        return self.grad[self.offsets[name][0]:]

    def load_parameters(self, w):
        """Set the FP32 master weights (flat, layer by layer) and their BF16 copy."""
        self.w.copy_(torch.as_tensor(w, dtype=torch.float32))
        self.w_bf.copy_(self.w.to(torch.bfloat16))

    # forward ------------------------------------------------------------------------------------
    def _conv(self, name, grid, x, out_bf=None, out_f=None, in_f32=False):
        _, cin, cout = self.offsets[name]
        relu = dict((n, r) for n, _, _, r in LAYERS)[name]
        call("pmg_nn_conv3d_forward", *grid, cin, cout, int(in_f32), x, self._w(name), self._b(name), int(relu),
             out_bf, out_f, stream())

    def forward(self):
        g1, g2, g3, st = self.g1, self.g2, self.g3, stream()
        self._conv("enc1a", g1, self.feat, self.a1)
        self._conv("enc1b", g1, self.a1, self.a2)
        call("pmg_nn_pool2", 0, *g2, 16, self.a2, self.p2, st)
        self._conv("enc2a", g2, self.p2, self.a3)
        self._conv("enc2b", g2, self.a3, self.a4)
        call("pmg_nn_pool2", 0, *g3, 32, self.a4, self.p3, st)
        self._conv("enc3a", g3, self.p3, self.a5)
        self._conv("enc3b", g3, self.a5, self.a6)
        call("pmg_nn_copy_channels", self.v2, 32, 96, 0, self.a4, self.cat2, st)
        call("pmg_nn_up2", 0, *g3, 64, 96, 32, self.a6, self.cat2, st)
        self._conv("dec2", g2, self.cat2, self.a7)
        call("pmg_nn_copy_channels", self.v1, 16, 48, 0, self.a2, self.cat1, st)
        call("pmg_nn_up2", 0, *g2, 32, 48, 16, self.a7, self.cat1, st)
        self._conv("dec1", g1, self.cat1, self.a8)
        self._conv("head", g1, self.a8, None, self.out)
        return self.out

    # backward -----------------------------------------------------------------------------------
    def _wgrad(self, name, grid, x, dout):
        _, cin, cout = self.offsets[name]
        call("pmg_nn_conv3d_backward_weights", *grid, cin, cout, 0, x, dout, self._g(name), 0, self.scratch, stream())

    def _dgrad(self, name, grid, dout, din):
        _, cin, cout = self.offsets[name]
        call("pmg_nn_conv3d_backward_data", *grid, cin, cout, dout, self._w(name), din, stream())

    def backward(self):
        g1, g2, g3, st = self.g1, self.g2, self.g3, stream()
        v1, v2, v3 = self.v1, self.v2, self.v3
        self._wgrad("head", g1, self.a8, self.d_out)
        self._dgrad("head", g1, self.d_out, self.d_a8)
        call("pmg_nn_relu_backward", v1 * 16, self.a8, self.d_a8, st)
        self._wgrad("dec1", g1, self.cat1, self.d_a8)
        self._dgrad("dec1", g1, self.d_a8, self.d_cat1)
        self.d_a2.zero_()
        call("pmg_nn_split_channels", v1, 16, 48, 0, self.d_cat1, self.d_a2, st)
        call("pmg_nn_up2", 1, *g2, 32, 48, 16, self.d_cat1, self.d_a7, st)
        call("pmg_nn_relu_backward", v2 * 32, self.a7, self.d_a7, st)
        self._wgrad("dec2", g2, self.cat2, self.d_a7)
        self._dgrad("dec2", g2, self.d_a7, self.d_cat2)
        self.d_a4.zero_()
        call("pmg_nn_split_channels", v2, 32, 96, 0, self.d_cat2, self.d_a4, st)
        call("pmg_nn_up2", 1, *g3, 64, 96, 32, self.d_cat2, self.d_a6, st)
        call("pmg_nn_relu_backward", v3 * 64, self.a6, self.d_a6, st)
        self._wgrad("enc3b", g3, self.a5, self.d_a6)
        self._dgrad("enc3b", g3, self.d_a6, self.d_a5)
        call("pmg_nn_relu_backward", v3 * 64, self.a5, self.d_a5, st)
        self._wgrad("enc3a", g3, self.p3, self.d_a5)
        self._dgrad("enc3a", g3, self.d_a5, self.d_p3)
        call("pmg_nn_pool2", 1, *g3, 32, self.d_p3, self.d_a4, st)     # adds into d_a4
        call("pmg_nn_relu_backward", v2 * 32, self.a4, self.d_a4, st)
        self._wgrad("enc2b", g2, self.a3, self.d_a4)
        self._dgrad("enc2b", g2, self.d_a4, self.d_a3)
        call("pmg_nn_relu_backward", v2 * 32, self.a3, self.d_a3, st)
        self._wgrad("enc2a", g2, self.p2, self.d_a3)
        self._dgrad("enc2a", g2, self.d_a3, self.d_p2)
        call("pmg_nn_pool2", 1, *g2, 16, self.d_p2, self.d_a2, st)     # adds into d_a2
        call("pmg_nn_relu_backward", v1 * 16, self.a2, self.d_a2, st)
        self._wgrad("enc1b", g1, self.a1, self.d_a2)
        self._dgrad("enc1b", g1, self.d_a2, self.d_a1)
        call("pmg_nn_relu_backward", v1 * 16, self.a1, self.d_a1, st)
        self._wgrad("enc1a", g1, self.feat, self.d_a1)
        return self.grad

    def state_dict(self):
        """FP32 master weights, their BF16 copy, Adam moments and step (checkpoint)."""
        return {"w": self.w, "w_bf": self.w_bf, "m": self.m, "v": self.v, "step_count": self.step_count}

    def load_state_dict(self, sd):
        for k in ("w", "w_bf", "m", "v"):
            getattr(self, k).copy_(sd[k].to(getattr(self, k).device))
        self.step_count = int(sd["step_count"])

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.step_count += 1
        call("pmg_nn_adam", self.nparam, self.w, self.grad, self.m, self.v, self.w_bf, lr, beta1, beta2, eps,
             self.step_count, weight_decay, stream())


class LearnedWarmStart:
    """Online-trained predictor of the displacement field for MixedPrecisionCG (`warm_start=`).

    grid: the fine element grid (nelx, nely, nelz) of the operator; the network works on the voxels of
    stride `stride` (a coarse multigrid level), its nodal output is prolongated to the fine grid by the
    multigrid prolongation.  observe() stores (features, normalised injected solution) pairs in a ring of
    `capacity` samples and takes `train_steps` Adam steps on them; predict() runs the network once the
    first `min_samples` pairs were seen.
    """

    def __init__(self, grid, stride=4, capacity=8, train_steps=2, lr=1e-3, min_samples=1, seed=0, device="cuda",
                 use_net=True, history=1, train_every=1, gate=0.0, gate_skip=3, coarse_correction=False):
        """train_every: train on every k-th observed solution (the pairs are stored every time).
        gate, gate_skip: when the network's prediction carried less than `gate` of the energy norm of the
        Rayleigh-Ritz initial guess, skip the next `gate_skip` predictions (then predict again); each further
        prediction below the gate in a row doubles the skip (at most 32) and the training interval (at most
        8 x train_every), a prediction above it resets both; gate 0 disables.
        coarse_correction: MixedPrecisionCG also uses the prediction w of a solve as a one-dimensional coarse
        space in every flexible-CG iteration, deflated (A-DEF2, Tang, Nabben, Vuik, Erlangga, J. Sci. Comput.
        39 (2009)): z = M(r - (w.r / w.Kw) Kw) + (w.r / w.Kw) w."""
        nx, ny, nz = grid
        self.use_net = use_net
        self.coarse_correction = bool(coarse_correction)
        self.train_every, self.gate, self.gate_skip = max(1, int(train_every)), float(gate), int(gate_skip)
        self._skip = 0
        self._fail = 0              # predictions below the gate in a row
        self._predicted = False
        self.predictions = 0
        self.history = int(history)
        self._hist = []             # older solutions (FP64, fine grid), most recent first
        if nz == 0:
            raise ValueError("the learned warm start is 3D")
        if nx % stride or ny % stride or nz % stride or stride & (stride - 1):
            raise ValueError("grid must be divisible by the stride (a power of two)")
        self.grid, self.stride = (nx, ny, nz), stride
        self.vgrid = (nx // stride, ny // stride, nz // stride)
        self.net = ConvNet3D(self.vgrid, device=device, seed=seed)
        self.capacity, self.train_steps, self.lr, self.min_samples = capacity, train_steps, lr, min_samples
        vx, vy, vz = self.vgrid
        self.ncn = (vx + 1) * (vy + 1) * (vz + 1) * 3          # coarse nodal dofs
        self.feats = torch.zeros((capacity, self.net.v1 * 4), dtype=torch.bfloat16, device=device)
        self.targets = torch.zeros((capacity, self.ncn), dtype=torch.float64, device=device)
        self.count = 0
        self.rng = np.random.default_rng(seed)
        f64 = dict(dtype=torch.float64, device=device)
        self._pred = torch.zeros(self.ncn, **f64)
        self._dpred = torch.zeros(self.ncn, dtype=torch.float32, device=device)
        self._loss = torch.zeros((self.ncn + 255) // 256, **f64)
        self._sc = torch.zeros(2, **f64)
        # prolongation chain buffers: stride s -> s/2 -> ... -> 1
        self._levels = []
        s = stride
        while s > 1:
            s //= 2
            g = (nx // s, ny // s, nz // s)
            self._levels.append((g, torch.zeros((g[0] + 1) * (g[1] + 1) * (g[2] + 1) * 3, **f64)))
        self.last_loss = None
        # training runs on a side stream (lower priority than the solver's) after the pair it learns from is
        # stored; the next forward pass waits for it
        self.side_stream = torch.cuda.Stream(device=device, priority=0) if str(device).startswith("cuda") else None
        self._trained = None

    def sync_training(self):
        """Order the current stream after the training steps issued so far."""
        if self._trained is not None:
            torch.cuda.current_stream().wait_event(self._trained)
            self._trained = None

    def state_dict(self):
        """Network, training buffer, sample count, random state, gate and history (checkpoint)."""
        self.sync_training()
        return {"net": self.net.state_dict(), "feats": self.feats, "targets": self.targets, "count": self.count,
                "rng": self.rng.bit_generator.state, "skip": self._skip, "fail": self._fail,
                "predictions": self.predictions,
                "hist": list(self._hist)}

    def load_state_dict(self, sd):
        self.sync_training()
        self.net.load_state_dict(sd["net"])
        self.feats.copy_(sd["feats"].to(self.feats.device))
        self.targets.copy_(sd["targets"].to(self.targets.device))
        self.count, self._skip, self.predictions = int(sd["count"]), int(sd["skip"]), int(sd["predictions"])
        self._fail = int(sd.get("fail", 0))
        self.rng.bit_generator.state = sd["rng"]
        self._hist = [h.to(self.targets.device) for h in sd["hist"]]

    @property
    def ready(self):
        return self.count >= self.min_samples

    def _features(self, xe64, out):
        nx, ny, nz = self.grid
        call("pmg_nn_input_features", nx, ny, nz, self.stride, *self.vgrid, xe64, out, stream())

    def predict(self, A):
        """FP64 prediction of the fine nodal displacement for the operator A (not masked, arbitrary scale)."""
        self.sync_training()
        self._features(A._xe64 if A._xe64 is not None else A.xe, self.net.feat)
        self.net.forward()
        call("pmg_nn_vox_to_node", 0, *self.vgrid, self.net.out, self._pred, stream())
        src, st = self._pred, stream()
        for g, buf in self._levels:
            buf.zero_()
            call("pmg_prolong_add", F64, g[0], g[1], g[2], src, buf, st)
            src = buf
        return src

    def basis(self, A, x0):
        """Directions of the Rayleigh-Ritz initial guess besides x0: the `history` solutions before the
        latest one (x0 is the latest, as LinSolve passes it; linear extrapolation in the design sequence)
        and the network's prediction."""
        hist = [h for h in self._hist if h.numel() == A.grid.ndof]
        vecs = hist[1:1 + self.history] if x0 is not None else hist[:self.history]
        self._predicted = False
        if self.use_net and self.ready:
            if self._skip > 0:
                self._skip -= 1
            else:
                vecs.append(self.predict(A))
                self._predicted = True
                self.predictions += 1
        return vecs

    def report(self, shares):
        """Energy shares of the Rayleigh-Ritz directions of the last solve (the prediction is the last one when
        it was used): a prediction below the gate suspends the next predictions (gate_skip, doubled for each
        further one below the gate in a row, at most 32)."""
        if not self._predicted or self.gate <= 0.0 or not len(shares):
            return
        if float(shares[-1]) < self.gate:
            self._fail += 1
            self._skip = min(32, self.gate_skip << min(self._fail - 1, 5))
        else:
            self._fail = 0

    def observe(self, A, u):
        """Store the pair (stiffness field of A, solution u) and train on the stored pairs (side stream)."""
        self.sync_training()          # the training buffer is written below; earlier steps may still read it
        if self.history > 0:
            keep = self._hist[:self.history + 1]
            buf = keep.pop() if len(keep) == self.history + 1 else torch.empty_like(u)
            buf.copy_(u)
            self._hist = [buf] + keep
        if not self.use_net:
            return
        slot = self.count % self.capacity
        self._features(A._xe64 if A._xe64 is not None else A.xe, self.feats[slot])
        t = self.targets[slot]
        nx, ny, nz = self.grid
        call("pmg_nn_inject", nx, ny, nz, self.stride, u, 1.0, t, stream())
        ws = _workspace(u.device)
        call("pmg_dot", F64, self.ncn, t, t, self._sc[0:1], ws.reduce, stream())
        call("pmg_scale_rsqrt", F64, self.ncn, t, t, self._sc[0:1], stream())   # unit 2-norm
        self.count += 1
        every = self.train_every << min(self._fail, 3)      # backs off while the predictions do not help
        if (self.count - 1) % every == 0 and self.train_steps > 0:
            slots = [int(self.rng.integers(min(self.count, self.capacity))) for _ in range(self.train_steps)]
            if self.side_stream is None:
                for sl in slots:
                    self.train_step(sl)
                return
            stored = torch.cuda.Event()
            stored.record()                             # the new pair is in the buffer
            if self._trained is not None:               # previous training steps (same network buffers)
                self.side_stream.wait_event(self._trained)
            self.side_stream.wait_event(stored)
            with torch.cuda.stream(self.side_stream):
                for sl in slots:
                    self.train_step(sl)
                self._trained = torch.cuda.Event()
                self._trained.record()

    def train_step(self, slot):
        net = self.net
        net.feat.copy_(self.feats[slot])
        net.forward()
        call("pmg_nn_vox_to_node", 0, *self.vgrid, net.out, self._pred, stream())
        call("pmg_nn_mse", self.ncn, self._pred, self.targets[slot], 1.0, self._dpred, self._loss, stream())
        call("pmg_nn_vox_to_node", 1, *self.vgrid, self._dpred, net.d_out, stream())
        net.backward()
        net.adam(lr=self.lr)

    def loss(self):
        """Sum of the squared errors of the last training step (host synchronisation)."""
        self.sync_training()
        return float(self._loss.sum().item())


def _workspace(device):
    from .operators import Workspace
    return Workspace.get(device)


def rayleigh_ritz(A, b, vectors, out_x, out_r, work, A32=None, work32=None):
    """x = sum c_i v_i minimising the energy error over span(vectors) (Galerkin: G c = h with
    G_ij = v_i^T A v_j, h_i = v_i^T b), and r = b - A x.  `work` holds one FP64 vector per basis vector.
    Returns the coefficients.  Linearly dependent directions are dropped.
    With A32 (the FP32 operator of the same matrix) and work32 (two FP32 vectors) the Gram products use the
    FP32 level-0 operator, and r = b - A x is one FP64 product: the coefficients carry the FP32 rounding
    of the products, the residual is the exact FP64 residual of the returned x."""
    n = b.numel()
    st = stream()
    ws = _workspace(b.device)
    k = len(vectors)
    for v, q in zip(vectors, work):
        if A32 is None:
            A.apply(MATVEC, v, out=q)
        else:
            u32, y32 = work32
            call("pmg_convert", F64, F32, n, v, u32, 1.0, st)
            A32.apply(MATVEC, u32, out=y32)
            call("pmg_convert", F32, F64, n, y32, q, 1.0, st)
    sc = torch.zeros(k * k + k, dtype=torch.float64, device=b.device)
    for i in range(k):
        for j in range(i, k):
            call("pmg_dot", F64, n, vectors[i], work[j], sc[i * k + j:i * k + j + 1], ws.reduce, st)
        call("pmg_dot", F64, n, vectors[i], b, sc[k * k + i:k * k + i + 1], ws.reduce, st)
    vals = sc.cpu().numpy()
    G = vals[:k * k].reshape(k, k)
    G = np.triu(G) + np.triu(G, 1).T
    h = vals[k * k:]
    keep = [i for i in range(k) if G[i, i] > 0 and np.isfinite(G[i, i])]
    c = np.zeros(k)
    if keep:
        Gk = G[np.ix_(keep, keep)]
        d = np.sqrt(np.diag(Gk))
        Gs = Gk / np.outer(d, d)
        w, V = np.linalg.eigh(Gs)
        good = w > 1e-10 * w.max()
        ck = (V[:, good] @ ((V[:, good].T @ (h[keep] / d)) / w[good])) / d
        c[keep] = ck
    out_x.zero_()
    for ci, v in zip(c, vectors):
        if ci != 0.0:
            out_x.add_(v, alpha=float(ci))
    if A32 is None:
        out_r.copy_(b)
        for ci, q in zip(c, work):
            if ci != 0.0:
                out_r.add_(q, alpha=-float(ci))
    else:
        A.apply(RESIDUAL, out_x, b, out=out_r)
    # energy share of each direction in the combination: |c_i| sqrt(G_ii) / sqrt(c^T G c)
    e = float(c @ G @ c) if keep else 0.0
    rayleigh_ritz.last_shares = (np.abs(c) * np.sqrt(np.maximum(np.diag(G), 0.0)) / np.sqrt(e)) if e > 0 else c * 0
    return c
