"""Learned-manifold hyper-reduced LSPG for the 2D shallow-water slip-wall
problem, and the affine (POD) LSPG it is compared against.

Offline: full-order snapshots come from the batched device FOM (one launch
per residual phase over all training parameter points, SSP-RK3 steps
replayed from a CUDA graph); the autoencoder is trained on the device by the
library (tcgen05 BF16 GEMMs, fp32 accumulation, Adam).  Online: hyper-reduced
LSPG (BDF1, Gauss-Newton, FP64 normal equations) on a sample mesh, with the
decoder evaluated only at the stencil-mesh rows.  Torch holds device buffers
and does the offline bookkeeping (slicing, normalisation, the POD basis of
the affine baseline); every residual, Jacobian, GEMM and solve runs in the
library's kernels.  The reference (pressio-demoapps) has no ROM; the LSPG
algorithm is Pressio's (rom/impl/lspg_unsteady_rj_policy_hypred.hpp), with
BDF1 or BDF2.  The full-order model is the ROM's fallback (FallbackRun).
"""
from __future__ import annotations

import time

import numpy as np

SWE_RANGES = {"gravity": (5.0, 10.0), "coriolis": (-4.0, -1.0), "pulseMagnitude": (0.05, 0.2)}


def latin_hypercube(n, ranges=SWE_RANGES, seed=0):
    """n points, one per stratum in every coordinate (seeded)."""
    rng = np.random.default_rng(seed)
    names = list(ranges)
    pts = []
    cols = {}
    for name in names:
        lo, hi = ranges[name]
        u = (rng.permutation(n) + rng.uniform(0, 1, n)) / n
        cols[name] = lo + u * (hi - lo)
    for i in range(n):
        pts.append({name: float(cols[name][i]) for name in names})
    return pts


def uniform_points(n, ranges=SWE_RANGES, seed=1):
    rng = np.random.default_rng(seed)
    return [{k: float(rng.uniform(*ranges[k])) for k in ranges} for _ in range(n)]


class SweSetup:
    """Full mesh [-5,5]^2 n x n (stencil 7), WENO5 slip-wall problems."""

    def __init__(self, pda, n=256, stream=None):
        import torch
        self.pda, self.n = pda, n
        self.stream = stream or torch.cuda.Stream()
        self.mesh = pda.create_full_mesh((n, n), (-5.0, 5.0, -5.0, 5.0), 7)
        self.N = 3 * n * n
        self.uref = torch.zeros(self.N, dtype=torch.float64, device="cuda")
        self.uref[0::3] = 1.0

    def problem(self, params, mesh=None):
        pda = self.pda
        return pda.create_problem(mesh or self.mesh, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 1,
                                  params, stream=self.stream)

    def snapshots(self, params_list, dt, n_steps, every=1):
        """FP32 states after every `every` steps (steps 1..n_steps), shape
        [points, n_steps // every, N], from one batched FOM run."""
        import torch
        probs = [self.problem(p) for p in params_list]
        B = self.pda.create_batch(probs, stream=self.stream)
        U = B.initialCondition()
        ns = n_steps // every
        S = torch.empty(len(params_list), ns, self.N, dtype=torch.float32, device="cuda")
        off = B.offsets
        for s in range(ns):
            B.advance_ssprk3(U, 0.0, dt, every)
            self.stream.synchronize()
            for i in range(len(params_list)):
                S[i, s] = U[off[i]: off[i] + self.N].float()
        return S

    def fom_trajectory(self, params, dt, checkpoints):
        """Single-problem FOM (SSP-RK3, CUDA-graph steps); returns the states
        at the checkpoint step counts and the wall time of the whole run."""
        p = self.problem(params)
        U = p.initialCondition()
        p.advance_ssprk3(U, 0.0, dt, 1)  # capture the step graph (excluded below)
        U = p.initialCondition()
        self.stream.synchronize()
        states, done, wall = {}, 0, 0.0
        for c in sorted(checkpoints):
            t0 = time.perf_counter()
            p.advance_ssprk3(U, 0.0, dt, c - done)
            self.stream.synchronize()
            wall += time.perf_counter() - t0
            done = c
            states[c] = U.clone()
        return states, wall

    def normalization(self, S):
        """uref = (1, 0, 0) per cell; scale per field = max |u - uref| over the
        snapshots (a floor keeps it positive)."""
        import torch
        scale = torch.empty(self.N, dtype=torch.float64, device="cuda")
        ref = self.uref.float()
        for d in range(3):
            m = (S[:, :, d::3] - ref[d::3]).abs().max().item()
            scale[d::3] = max(m, 1e-8)
        return scale

    def training_data(self, S, scale):
        """bf16 rows (u - uref) / scale, [points * snapshots, N]."""
        import torch
        X = torch.empty(S.shape[0] * S.shape[1], self.N, dtype=torch.bfloat16, device="cuda")
        ref, sc = self.uref.float(), scale.float()
        for i in range(S.shape[0]):
            X[i * S.shape[1]:(i + 1) * S.shape[1]] = ((S[i] - ref) / sc).to(torch.bfloat16)
        return X

    def sample_mesh(self, frac=0.01, seed=0):
        """frac of the cells with a fixed seed, plus their WENO5 stencils."""
        rng = np.random.default_rng(seed)
        ncell = self.n * self.n
        gids = np.sort(rng.choice(ncell, max(1, int(round(frac * ncell))), replace=False))
        sm, st = self.pda.create_sample_mesh(self.mesh, gids)
        s2st = np.searchsorted(st, gids)
        return sm, gids, st, s2st


def train_schedule(ae, X, epochs, batch=256, lr=1e-3, seed=2):
    """Adam in three phases of decreasing step size (60 % of the epochs at lr,
    25 % at lr / 3, 15 % at lr / 10); returns the per-epoch losses."""
    e1 = max(1, int(round(0.6 * epochs)))
    e2 = max(0, int(round(0.25 * epochs)))
    e3 = max(0, epochs - e1 - e2)
    out = [ae.train(X, batch=batch, epochs=e1, lr=lr, seed=seed)]
    if e2:
        out.append(ae.train(X, batch=batch, epochs=e2, lr=lr / 3, seed=seed + 1))
    if e3:
        out.append(ae.train(X, batch=batch, epochs=e3, lr=lr / 10, seed=seed + 2))
    return np.concatenate(out)


def stencil_rows(stencil_gids):
    st = np.asarray(stencil_gids, dtype=np.int64)
    return (st[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)


def pod_basis(S, uref, k):
    """Leading k left singular vectors of the snapshots minus uref (randomised
    SVD, float32), as float64 [N x k]."""
    import torch
    A = (S.reshape(-1, S.shape[-1]) - uref.float()).T  # N x ns
    U, _, _ = torch.svd_lowrank(A, q=k + 8, niter=4)
    return U[:, :k].double().contiguous()


class LearnedRom:
    """Autoencoder + LSPG construction for one sample mesh."""

    def __init__(self, setup, ae, scale):
        self.setup, self.ae, self.scale = setup, ae, scale
        import torch
        # the weights the network was trained with: bf16 values of the fp32 masters
        self.dec = tuple(t.to(torch.bfloat16).float() if t.dim() == 2 else t for t in ae.decoder())

    def encode(self, U):
        import torch
        x = ((U - self.setup.uref) / self.scale).float().to(torch.bfloat16).reshape(1, -1)
        _, Z = self.ae.reconstruct(x.contiguous())
        return Z[0].double().contiguous()

    def lspg(self, problem, s2st, stencil_gids, tensor_cores=True, jacobian_bits=32):
        """tensor_cores: the decoder's output layer as a bf16 tcgen05 GEMM (the
        numerics the network was trained with); False: fp32 on CUDA cores.
        jacobian_bits: 32 forms the Gauss-Newton Jacobian terms in single
        precision (the residual and normal equations stay double), 64 exactly."""
        rows = stencil_rows(stencil_gids)
        import torch
        r = torch.from_numpy(rows).cuda()
        W1, b1, W2, b2, W3, b3 = self.dec
        rom = self.setup.pda.LspgRom.mlp(problem, s2st, self.setup.uref[r].contiguous(),
                                         self.scale[r].contiguous(), W1, b1, W2, b2, W3[r].contiguous(),
                                         b3[r].contiguous(), tensor_cores=tensor_cores)
        rom.set_jacobian_precision(jacobian_bits)
        return rom

    def full_decoder(self):
        """The decoder on every row (error evaluation), through a full-mesh LSPG object."""
        s = self.setup
        p = s.problem({"gravity": 9.8, "coriolis": -3.0, "pulseMagnitude": 0.125})
        ident = np.arange(s.n * s.n)
        W1, b1, W2, b2, W3, b3 = self.dec
        return s.pda.LspgRom.mlp(p, ident, s.uref, self.scale, W1, b1, W2, b2, W3, b3), p


def affine_lspg(setup, phi, problem, s2st, stencil_gids, jacobian_bits=32):
    import torch
    r = torch.from_numpy(stencil_rows(stencil_gids)).cuda()
    rom = setup.pda.LspgRom.affine(problem, s2st, setup.uref[r].contiguous(), phi[r].contiguous())
    rom.set_jacobian_precision(jacobian_bits)
    return rom


def rel_l2(a, b, ref=None):
    import torch
    num = torch.linalg.vector_norm(a - b).item()
    den = torch.linalg.vector_norm(b if ref is None else b - ref).item()
    return num / max(den, 1e-300)


def run_rom(rom, x0, dt, checkpoints_steps, stream, gn_iters=5, tol=1e-9, order=1):
    """Advance the latent through the checkpoints (step counts of size dt)
    with BDF1 (order 1) or BDF2 (order 2); returns {step: latent}, wall
    seconds, max residual norm.  The step graphs are captured on the buffer
    the timed run uses, so no capture or instantiation is timed."""
    import torch
    x = x0.clone()
    rom.advance(x, dt, 1, gn_iters, tol, order=order, first_step=1)  # capture the first step's graph
    if order == 2:
        rom.advance(x, dt, 1, gn_iters, tol, order=2, first_step=2)  # and the BDF2 step's
    with torch.cuda.stream(stream):
        x.copy_(x0)
    stream.synchronize()
    out, done, wall, maxres = {}, 0, 0.0, 0.0
    for c in sorted(checkpoints_steps):
        t0 = time.perf_counter()
        info = rom.advance(x, dt, c - done, gn_iters, tol, order=order, first_step=done + 1)
        wall += time.perf_counter() - t0
        maxres = max(maxres, info["max_residual"])
        done = c
        out[c] = x.clone()
    return out, wall, maxres


class FallbackRun:
    """A ROM trajectory whose steps fall back to the full-order model.

    The ROM advances checkpoint by checkpoint; when the largest Gauss-Newton
    residual norm of a stretch exceeds `threshold`, that stretch is dropped,
    the latent state at its start is decoded to the full state and the GPU FOM
    (SSP-RK3 at the FOM step) advances from there to the end.  `states` holds
    the full state at every checkpoint (decoded where the ROM produced it),
    `fallback_at` the FOM step count where the FOM took over (None if never)."""

    def __init__(self, setup, params, rom, decoder, x0, dt_fom, ratio, checkpoints, threshold, gn_iters=1,
                 tol=1e-9, order=1):
        import torch
        if any(c % ratio for c in checkpoints):
            raise ValueError(f"every checkpoint must be a multiple of the ROM step ratio {ratio}: {checkpoints}")
        self.states, self.fallback_at = {}, None
        x = x0.clone()
        rom.advance(x, dt_fom * ratio, 1, gn_iters, tol, order=order, first_step=1)
        if order == 2:
            rom.advance(x, dt_fom * ratio, 1, gn_iters, tol, order=2, first_step=2)
        with torch.cuda.stream(setup.stream):
            x.copy_(x0)
        fom = setup.problem(params)
        U = fom.initialCondition()
        fom.advance_ssprk3(U, 0.0, dt_fom, 1)  # capture the FOM step graph on U
        setup.stream.synchronize()
        wall, done = 0.0, 0
        for c in sorted(checkpoints):
            t0 = time.perf_counter()
            if self.fallback_at is None:
                with torch.cuda.stream(setup.stream):
                    start = x.clone()
                info = rom.advance(x, dt_fom * ratio, (c - done) // ratio, gn_iters, tol, order=order,
                                   first_step=done // ratio + 1)
                if info["max_residual"] > threshold:
                    self.fallback_at = done
                    y = decoder.decode(start)
                    with torch.cuda.stream(setup.stream):
                        U.copy_(y)
                    fom.advance_ssprk3(U, done * dt_fom, dt_fom, c - done)
            else:
                fom.advance_ssprk3(U, done * dt_fom, dt_fom, c - done)
            setup.stream.synchronize()
            wall += time.perf_counter() - t0
            self.states[c] = U.clone() if self.fallback_at is not None else decoder.decode(x)
            done = c
        self.wall = wall


def timed(fn):
    t0 = time.perf_counter()
    r = fn()
    return r, time.perf_counter() - t0
