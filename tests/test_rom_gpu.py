"""Learned-manifold ROM pieces on the GPU against the CPU oracles:

* autoencoder gradients (tcgen05 BF16 GEMMs, fp32 accumulation) against
  oracle/mlp_oracle.py replaying the same bf16 roundings in float64 --
  tolerance: per layer ||g - g_ref|| <= 3e-2 ||g_ref|| (the device accumulates
  in fp32 and a bf16 rounding on either side may land one bf16 ulp apart), loss
  within 1e-3;
* training lowers the loss on a low-rank data set;
* hyper-reduced LSPG (BDF1, Gauss-Newton) with an affine basis and with an MLP
  decoder against oracle/lspg_oracle.py on the same sample-mesh problem --
  latent trajectories within 1e-8 relative (FP64 on both sides, different
  summation orders in J D and the normal equations); graph replay equals the
  eager path bit for bit."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ORACLE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
sys.path.insert(0, ORACLE)


def _bf16(torch, a):
    return torch.from_numpy(np.asarray(a, dtype=np.float32)).cuda().to(torch.bfloat16)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [192, 4096])
def test_autoencoder_gradients_match_oracle(pda, n):
    """n = 4096: the wide layers' blocked-operand GEMMs split K over CTAs."""
    import torch
    import mlp_oracle
    k, ha, hb, B = 4, 128, 64, 64
    ae = pda.AutoEncoder(n, k, ha, hb, seed=3)
    rng = np.random.default_rng(5)
    X = rng.normal(0, 0.5, (B, n))
    Xd = _bf16(torch, X)
    loss, g = ae.gradients(Xd)
    Ws, bs = [], []
    for l in range(6):
        W, b = ae.layer(l)
        Ws.append(W.double().cpu().numpy())
        bs.append(b.double().cpu().numpy())
    lref, gW, gb = mlp_oracle.loss_and_gradients(Ws, bs, Xd.float().cpu().numpy(), bf16=True)
    assert abs(loss - lref) <= 1e-3 * lref
    g = g.double().cpu().numpy()
    off = 0
    for l in range(6):
        o, i = Ws[l].shape
        gw = g[off: off + o * i].reshape(o, i)
        off += o * i
        gbb = g[off: off + o]
        off += o
        for got, ref in ((gw, gW[l]), (gbb, gb[l])):
            nr = np.linalg.norm(ref)
            if nr == 0:
                assert np.linalg.norm(got) == 0
            else:
                assert np.linalg.norm(got - ref) <= 3e-2 * nr, (l, np.linalg.norm(got - ref) / nr)


@pytest.mark.gpu
def test_autoencoder_training_reduces_loss(pda):
    import torch
    n, k = 256, 4
    rng = np.random.default_rng(0)
    basis = rng.normal(0, 1, (3, n))
    coef = rng.uniform(-1, 1, (1024, 3))
    X = np.tanh(0.5 * coef @ basis)
    ae = pda.AutoEncoder(n, k, 256, 128, seed=1)
    losses = ae.train(_bf16(torch, X), batch=128, epochs=60, lr=2e-3, seed=2)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.1 * losses[0], losses[[0, -1]]
    Y, Z = ae.reconstruct(_bf16(torch, X[:200]))
    err = np.linalg.norm(Y.cpu().numpy() - X[:200]) / np.linalg.norm(X[:200])
    assert err < 0.2, err
    assert Z.shape == (200, k)


@pytest.mark.gpu
def test_autoencoder_fused_adam_equals_separate_pass(pda):
    """Adam inside the weight-gradient GEMM epilogues (with the bf16 copy and
    transpose refreshed there) and Adam as a separate pass over stored
    gradients give the same weights, biases and losses bit for bit; the
    latent padding stays zero."""
    import torch
    n, k, ha, hb = 384, 5, 256, 128
    rng = np.random.default_rng(7)
    X = _bf16(torch, np.tanh(rng.normal(0, 0.7, (512, 3)) @ rng.normal(0, 1, (3, n))))
    out = []
    for fused in (True, False):
        ae = pda.AutoEncoder(n, k, ha, hb, seed=4)
        ae.set_fused(fused)
        losses = ae.train(X, batch=128, epochs=3, lr=3e-3, seed=9)
        out.append((losses, [tuple(t.cpu().numpy() for t in ae.layer(l)) for l in range(6)]))
    (la, wa), (lb, wb) = out
    assert np.array_equal(la, lb), (la, lb)
    for l in range(6):
        assert np.array_equal(wa[l][0], wb[l][0]) and np.array_equal(wa[l][1], wb[l][1]), l
    assert np.all(wa[2][0][k:] == 0) and np.all(wa[2][1][k:] == 0)  # encoder output rows past the latent
    assert np.all(wa[3][0][:, k:] == 0)  # decoder input columns past the latent
    assert la[-1] < la[0]


def _sample_problem(pda, oracle, n=24, frac=0.3, seed=0):
    full = pda.create_full_mesh((n, n), (-5, 5, -5, 5), 7, (False, False))
    rng = np.random.default_rng(seed)
    gids = np.sort(rng.choice(n * n, int(frac * n * n), replace=False))
    sm, st = pda.create_sample_mesh(full, gids)
    params = {"gravity": 7.0, "coriolis": -2.0, "pulseMagnitude": 0.15}
    import torch
    stream = torch.cuda.Stream()
    ps = pda.create_problem(sm, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 1, params, stream=stream)
    g, x, y, z, _, _ = sm._arrays()
    om = oracle.mesh_from_arrays(2, 7, g, x, y, z, (sm.dx(), sm.dy(), sm.dz()))
    po = oracle.problem(om, 3, 0, 2, 1, params)
    s2st = np.searchsorted(st, gids)
    return full, sm, st, ps, po, om, s2st, rng


@pytest.mark.gpu
def test_lspg_affine_matches_oracle_and_graph(pda, oracle):
    import torch
    import lspg_oracle
    full, sm, st, ps, po, om, s2st, rng = _sample_problem(pda, oracle)
    nst = len(st) * 3
    k = 6
    uref = np.zeros(nst)
    uref[0::3] = 1.0
    phi, _ = np.linalg.qr(rng.normal(0, 1, (nst, k)))
    phi *= 0.3
    x0 = np.array([0.1, -0.05, 0.02, 0.0, 0.01, -0.02])
    dt, steps = 0.01, 4
    xr, traj = lspg_oracle.lspg_bdf1(po, s2st, lspg_oracle.affine_decoder(uref, phi), x0, dt, steps, iters=8,
                                     tol=1e-12)
    rom = pda.LspgRom.affine(ps, s2st, torch.from_numpy(uref).cuda(), torch.from_numpy(phi).cuda())
    xd = torch.from_numpy(x0).cuda()
    info = rom.advance_bdf1(xd, dt, steps, gn_iters=8, tol=1e-12, use_graph=False)
    assert np.allclose(xd.cpu().numpy(), xr, rtol=1e-8, atol=1e-12), (xd.cpu().numpy(), xr)
    assert info["iters_last_step"] >= 1
    xg = torch.from_numpy(x0).cuda()
    rom.advance_bdf1(xg, dt, steps, gn_iters=8, tol=1e-12, use_graph=True)
    assert torch.equal(xg, xd)
    y = rom.decode(xd)
    assert np.allclose(y.cpu().numpy(), uref + phi @ xd.cpu().numpy(), rtol=0, atol=1e-14)


@pytest.mark.gpu
def test_lspg_mlp_decoder_matches_oracle(pda, oracle):
    import torch
    import lspg_oracle
    full, sm, st, ps, po, om, s2st, rng = _sample_problem(pda, oracle, seed=1)
    nst = len(st) * 3
    k, h1, h2 = 4, 256, 128
    W1 = rng.normal(0, 0.5, (h1, k)).astype(np.float32)
    b1 = rng.normal(0, 0.1, h1).astype(np.float32)
    W2 = rng.normal(0, 0.1, (h2, h1)).astype(np.float32)
    b2 = rng.normal(0, 0.1, h2).astype(np.float32)
    W3 = rng.normal(0, 0.1, (nst, h2)).astype(np.float32)
    b3 = rng.normal(0, 0.1, nst).astype(np.float32)
    uref = np.zeros(nst)
    uref[0::3] = 1.0
    scale = np.full(nst, 0.05)
    ts = [torch.from_numpy(a).cuda() for a in (W1, b1, W2, b2, W3, b3)]
    rom = pda.LspgRom.mlp(ps, s2st, torch.from_numpy(uref).cuda(), torch.from_numpy(scale).cuda(), *ts)
    x0 = np.array([0.2, -0.1, 0.05, 0.1])
    # the decoder: float32 on the device, float64 in the oracle
    y = rom.decode(torch.from_numpy(x0).cuda()).cpu().numpy()
    dec = lspg_oracle.mlp_decoder(uref, scale, *[a.astype(np.float64) for a in (W1, b1, W2, b2, W3, b3)])
    yref, _ = dec(x0)
    assert np.max(np.abs(y - yref)) <= 1e-6 * np.max(np.abs(yref - uref))
    dt, steps = 0.01, 3
    xr, _ = lspg_oracle.lspg_bdf1(po, s2st, dec, x0, dt, steps, iters=8, tol=1e-10)
    xd = torch.from_numpy(x0).cuda()
    rom.advance_bdf1(xd, dt, steps, gn_iters=8, tol=1e-10, use_graph=True)
    # float32 decoder evaluation: the latent agrees to the decoder's precision
    assert np.allclose(xd.cpu().numpy(), xr, rtol=1e-4, atol=1e-6), (xd.cpu().numpy(), xr)


@pytest.mark.gpu
def test_lspg_mlp_tensor_core_decoder_close_to_fp32(pda, oracle):
    """Tensor-core output layer (bf16 weights and activations, fp32
    accumulation: the autoencoder's training numerics) against the fp32
    decoder: decoded states within 1e-2 of the perturbation scale, latent
    trajectories within 2e-2."""
    import torch
    full, sm, st, ps, po, om, s2st, rng = _sample_problem(pda, oracle, seed=2)
    nst = len(st) * 3
    k, h1, h2 = 4, 256, 128
    def bf(a):
        return torch.from_numpy(a.astype(np.float32)).cuda().to(torch.bfloat16).float()
    W1, W2, W3 = bf(rng.normal(0, 0.5, (h1, k))), bf(rng.normal(0, 0.1, (h2, h1))), bf(rng.normal(0, 0.1, (nst, h2)))
    b1, b2, b3 = (torch.from_numpy(rng.normal(0, 0.1, m).astype(np.float32)).cuda() for m in (h1, h2, nst))
    uref = np.zeros(nst)
    uref[0::3] = 1.0
    ur, sc = torch.from_numpy(uref).cuda(), torch.full((nst,), 0.05, dtype=torch.float64, device="cuda")
    r32 = pda.LspgRom.mlp(ps, s2st, ur, sc, W1, b1, W2, b2, W3, b3, tensor_cores=False)
    rtc = pda.LspgRom.mlp(ps, s2st, ur, sc, W1, b1, W2, b2, W3, b3, tensor_cores=True)
    x0 = torch.tensor([0.2, -0.1, 0.05, 0.1], dtype=torch.float64, device="cuda")
    y32, ytc = r32.decode(x0), rtc.decode(x0)
    pert = (y32 - ur).abs().max().item()
    assert (ytc - y32).abs().max().item() <= 1e-2 * pert
    xa, xb = x0.clone(), x0.clone()
    r32.advance_bdf1(xa, 0.01, 3, 6, 1e-10)
    rtc.advance_bdf1(xb, 0.01, 3, 6, 1e-10)
    assert torch.allclose(xa, xb, rtol=2e-2, atol=1e-3), (xa, xb)
    with pytest.raises(pda.PdaError):  # non-bf16 weights are refused in tensor-core mode
        pda.LspgRom.mlp(ps, s2st, ur, sc, W1, b1, W2, b2, W3 + 1e-4, b3, tensor_cores=True)


@pytest.mark.gpu
@pytest.mark.parametrize("family,problem,scheme,ic,params", [
    ("Swe2d", 0, 2, 1, {"gravity": 7.0, "coriolis": -2.0, "pulseMagnitude": 0.15}),
    ("Euler2d", 4, 1, 2, None),
    ("Euler2d", 3, 0, 1, None),
    ("Euler2d", 7, 2, 1, None),
])
def test_lspg_fused_iteration_equals_assembled_jacobian(pda, family, problem, scheme, ic, params):
    """The fused Gauss-Newton iteration (velocity and Jf D face by face, one
    launch) and the assembled path (CSR Jf, then Jf D) are the same LSPG
    iteration: latent trajectories agree to 1e-10 relative, on inner and
    near-boundary rows (Neumann mirrors, Sedov symmetry planes, cross-shock
    inflow states) of WENO5, WENO3 and first-order problems."""
    import torch
    n = 20
    bounds = (-5, 5, -5, 5) if family == "Swe2d" else ((0, 1.2, 0, 1.2) if problem == 3 else (0, 2, 0, 1))
    full = pda.create_full_mesh((n, n), bounds, 7)
    rng = np.random.default_rng(11)
    gids = np.sort(rng.choice(n * n, 90, replace=False))
    sm, st = pda.create_sample_mesh(full, gids)
    enum = getattr(pda, family)(problem)
    ps = pda.create_problem(sm, enum, pda.InviscidFluxReconstruction(scheme), ic, params)
    s2st = np.searchsorted(st, gids)
    nd = ps.numDofPerCell()
    nst = len(st) * nd
    pf = pda.create_problem(full, enum, pda.InviscidFluxReconstruction(scheme), ic, params)
    u0 = pf.initialCondition().cpu().numpy().reshape(-1, nd)[st].reshape(-1)
    k = 6
    phi, _ = np.linalg.qr(rng.normal(0, 1, (nst, k)))
    phi *= 0.5 * np.abs(u0)[:, None]  # relative perturbations keep pressures positive
    x0 = rng.normal(0, 0.05, k)
    out = []
    for fused in (True, False):
        rom = pda.LspgRom.affine(ps, s2st, torch.from_numpy(u0).cuda(), torch.from_numpy(phi).cuda())
        rom.set_fused(fused)
        x = torch.from_numpy(x0.copy()).cuda()
        rom.advance_bdf1(x, 0.002, 3, gn_iters=4, tol=0.0, use_graph=fused)
        out.append(x.cpu().numpy())
    assert np.all(np.isfinite(out[0]))
    assert np.allclose(out[0], out[1], rtol=1e-10, atol=1e-12 * np.max(np.abs(out[1]))), out


@pytest.mark.gpu
@pytest.mark.parametrize("family,problem,scheme,ic,params", [
    ("Swe2d", 0, 2, 1, {"gravity": 7.0, "coriolis": -2.0, "pulseMagnitude": 0.15}),
    ("Euler2d", 4, 1, 2, None),
    ("Euler2d", 3, 0, 1, None),
    ("Euler2d", 7, 2, 1, None),
])
def test_lspg_single_precision_jacobian_is_an_inexact_gauss_newton_step(pda, family, problem, scheme, ic, params):
    """Jacobian terms in single precision (reconstruction gradients, flux
    Jacobians, Jf D) with the residual, normal equations and solve in double.
    The single-precision Jacobian moves the Gauss-Newton fixed point (where
    J^T R = 0) by about its rounding error (6e-8) times the conditioning of
    the normal equations: the latent trajectories of 3 steps x 4 iterations
    agree with the exact Jacobian's to 2e-5 of the largest latent coordinate
    (measured: up to 4.3e-6 on these problems)."""
    import torch
    n = 20
    bounds = (-5, 5, -5, 5) if family == "Swe2d" else ((0, 1.2, 0, 1.2) if problem == 3 else (0, 2, 0, 1))
    full = pda.create_full_mesh((n, n), bounds, 7)
    rng = np.random.default_rng(12)
    gids = np.sort(rng.choice(n * n, 90, replace=False))
    sm, st = pda.create_sample_mesh(full, gids)
    enum = getattr(pda, family)(problem)
    ps = pda.create_problem(sm, enum, pda.InviscidFluxReconstruction(scheme), ic, params)
    s2st = np.searchsorted(st, gids)
    nd = ps.numDofPerCell()
    nst = len(st) * nd
    pf = pda.create_problem(full, enum, pda.InviscidFluxReconstruction(scheme), ic, params)
    u0 = pf.initialCondition().cpu().numpy().reshape(-1, nd)[st].reshape(-1)
    k = 6
    phi, _ = np.linalg.qr(rng.normal(0, 1, (nst, k)))
    phi *= 0.5 * np.abs(u0)[:, None]
    x0 = rng.normal(0, 0.05, k)
    out, info = [], []
    for bits in (64, 32):
        rom = pda.LspgRom.affine(ps, s2st, torch.from_numpy(u0).cuda(), torch.from_numpy(phi).cuda())
        rom.set_jacobian_precision(bits)
        x = torch.from_numpy(x0.copy()).cuda()
        info.append(rom.advance_bdf1(x, 0.002, 3, gn_iters=4, tol=0.0))
        out.append(x.cpu().numpy())
    assert np.all(np.isfinite(out[1]))
    scale = np.max(np.abs(out[0]))
    dev = np.max(np.abs(out[1] - out[0])) / scale
    assert dev <= 2e-5, (dev, out)
    assert not np.array_equal(out[1], out[0])  # the single-precision kernel ran
    with pytest.raises(pda.PdaError):
        rom.set_jacobian_precision(16)


@pytest.mark.gpu
def test_lspg_bdf2_matches_oracle_fused_assembled_graph_and_chunks(pda, oracle):
    """BDF2 LSPG (Pressio's hyper-reduced policy: step 1 with BDF1, then
    R = -2/3 dt V + (y - 4/3 y_n + 1/3 y_n-1)) against the numpy oracle:
    fused and assembled iterations, eager and graph replay, one call and the
    same steps split over calls that continue the step numbering."""
    import torch
    import lspg_oracle
    full, sm, st, ps, po, om, s2st, rng = _sample_problem(pda, oracle, seed=4)
    nst = len(st) * 3
    k = 6
    uref = np.zeros(nst)
    uref[0::3] = 1.0
    phi, _ = np.linalg.qr(rng.normal(0, 1, (nst, k)))
    phi *= 0.3
    x0 = np.array([0.1, -0.05, 0.02, 0.0, 0.01, -0.02])
    dt, steps = 0.01, 5
    xr, _ = lspg_oracle.lspg_bdf(po, s2st, lspg_oracle.affine_decoder(uref, phi), x0, dt, steps, order=2, iters=8,
                                 tol=1e-12)
    x1, _ = lspg_oracle.lspg_bdf1(po, s2st, lspg_oracle.affine_decoder(uref, phi), x0, dt, steps, iters=8,
                                  tol=1e-12)
    assert not np.allclose(xr, x1, rtol=1e-6)  # the second-order steps differ from BDF1's
    res = []
    for fused in (True, False):
        for graph in (False, True):
            rom = pda.LspgRom.affine(ps, s2st, torch.from_numpy(uref).cuda(), torch.from_numpy(phi).cuda())
            rom.set_fused(fused)
            x = torch.from_numpy(x0).cuda()
            rom.advance(x, dt, steps, gn_iters=8, tol=1e-12, order=2, first_step=1, use_graph=graph)
            res.append(x.cpu().numpy())
            assert np.allclose(res[-1], xr, rtol=1e-8, atol=1e-12), (fused, graph, res[-1], xr)
            # the same trajectory in three calls
            x = torch.from_numpy(x0).cuda()
            rom.advance(x, dt, 1, gn_iters=8, tol=1e-12, order=2, first_step=1, use_graph=graph)
            rom.advance(x, dt, 3, gn_iters=8, tol=1e-12, order=2, first_step=2, use_graph=graph)
            rom.advance(x, dt, 1, gn_iters=8, tol=1e-12, order=2, first_step=5, use_graph=graph)
            assert np.array_equal(x.cpu().numpy(), res[-1])
    assert np.array_equal(res[0], res[1]) and np.array_equal(res[2], res[3])


def _small_swe_rom(pda, n=24, k=6, seed=0):
    """A small slip-wall shallow-water ROM setup: full problem, sample mesh
    (30 % of the cells + WENO5 stencils), a POD basis of FOM snapshots, the
    sample LSPG and the full-mesh decoder of the same basis."""
    import torch
    import importlib.util
    spec = importlib.util.spec_from_file_location("pda_gb300_rom", os.path.join(
        os.path.dirname(ORACLE), "pressio-demoapps_gb300", "rom.py"))
    R = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(R)
    setup = R.SweSetup(pda, n)
    params = {"gravity": 7.5, "coriolis": -2.5, "pulseMagnitude": 0.15}
    dt = 0.01
    S = setup.snapshots([params], dt, 40)
    phi = R.pod_basis(S, setup.uref, k)
    sm, gids, st, s2st = setup.sample_mesh(0.3, seed=seed)
    ps = setup.problem(params, mesh=sm)
    rom = R.affine_lspg(setup, phi, ps, s2st, st, jacobian_bits=64)
    fp = setup.problem(params)
    dec = pda.LspgRom.affine(fp, np.arange(n * n), setup.uref, phi)
    U0 = fp.initialCondition()
    x0 = (phi.T @ (U0 - setup.uref)).contiguous()
    return R, setup, params, dt, rom, dec, x0


@pytest.mark.gpu
def test_rom_falls_back_to_the_fom(pda):
    """FallbackRun: with a residual threshold of 0 the first stretch's
    residual exceeds it, so the FOM takes over from the decoded initial
    latent and every checkpoint equals the FOM advanced from that state; with
    an infinite threshold the ROM runs to the end and matches run_rom."""
    import torch
    R, setup, params, dt, rom, dec, x0 = _small_swe_rom(pda)
    ratio, cps = 2, [4, 8, 12]
    fb = R.FallbackRun(setup, params, rom, dec, x0, dt, ratio, cps, threshold=0.0, gn_iters=2, order=2)
    assert fb.fallback_at == 0
    fom = setup.problem(params)
    U = dec.decode(x0)
    done = 0
    for c in cps:
        fom.advance_ssprk3(U, done * dt, dt, c - done)
        done = c
        setup.stream.synchronize()
        assert torch.equal(fb.states[c], U), c
    nofb = R.FallbackRun(setup, params, rom, dec, x0, dt, ratio, cps, threshold=float("inf"), gn_iters=2, order=2)
    assert nofb.fallback_at is None
    lat, _, _ = R.run_rom(rom, x0, dt * ratio, [c // ratio for c in cps], setup.stream, gn_iters=2, order=2)
    for c in cps:
        assert torch.equal(nofb.states[c], dec.decode(lat[c // ratio])), c


@pytest.mark.gpu
def test_learned_manifold_beats_linear_subspace(pda):
    """What the trained network gains over the method without it, at a
    reduced size (24 x 24 slip-wall shallow water, 6 training points x 60
    snapshots, latent 4): the autoencoder trained by the library's tcgen05
    kernels represents held-out FOM states (decoder(encoder(u))) more closely
    than the POD subspace of the same dimension built from the same
    snapshots."""
    import torch
    import importlib.util
    spec = importlib.util.spec_from_file_location("pda_gb300_rom", os.path.join(
        os.path.dirname(ORACLE), "pressio-demoapps_gb300", "rom.py"))
    R = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(R)
    n, k, dt = 24, 4, 0.01
    setup = R.SweSetup(pda, n)
    train = R.latin_hypercube(6, seed=3)
    S = setup.snapshots(train, dt, 60)
    scale = setup.normalization(S)
    X = setup.training_data(S, scale)
    phi = R.pod_basis(S, setup.uref, k)
    ae = pda.AutoEncoder(setup.N, k, 256, 256, seed=1, stream=setup.stream)
    R.train_schedule(ae, X, 200, batch=64, lr=2e-3, seed=2)
    learned = R.LearnedRom(setup, ae, scale)
    fdec, _ = learned.full_decoder()
    test = R.uniform_points(2, seed=9)
    e_ae, e_pod = [], []
    for p in test:
        states, _ = setup.fom_trajectory(p, dt, [20, 40, 60])
        for c in (20, 40, 60):
            u = states[c]
            e_ae.append(R.rel_l2(fdec.decode(learned.encode(u)), u, setup.uref))
            e_pod.append(R.rel_l2(setup.uref + phi @ (phi.T @ (u - setup.uref)), u, setup.uref))
    assert max(e_ae) < 0.5 and np.mean(e_ae) < 0.7 * np.mean(e_pod), (e_ae, e_pod)


LSPG_GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lspg")


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(f[:-4] for f in os.listdir(LSPG_GOLD) if f.endswith(".npz")))
@pytest.mark.parametrize("fused", [True, False])
def test_lspg_matches_pressio_golds(pda, name, fused):
    """The device LSPG (exact double Jacobian, fused and assembled iterations)
    reproduces the latent trajectories of the reference's own hyper-reduced
    LSPG -- vendored Pressio over the reference's slip-wall shallow-water
    problem on a reference-made sample mesh, BDF1 and BDF2
    (tests/golden/make_lspg_golden.py) -- step by step to 1e-8 relative."""
    import torch
    from conftest import mesh_dir
    g = dict(np.load(os.path.join(LSPG_GOLD, name + ".npz")))
    gr, co, pu = (float(v) for v in g["params"])
    sm = pda.load_cellcentered_uniform_mesh(mesh_dir("s2d_s7_20"))
    ps = pda.create_problem(sm, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 1,
                            {"gravity": gr, "coriolis": co, "pulseMagnitude": pu}, stream=torch.cuda.Stream())
    rom = pda.LspgRom.affine(ps, g["s2st"], torch.from_numpy(g["uref"]).cuda(), torch.from_numpy(g["phi"]).cuda())
    rom.set_fused(fused)
    rom.set_jacobian_precision(64)
    x = torch.from_numpy(g["x0"].copy()).cuda()
    scale = np.max(np.abs(g["traj"]))
    for n in range(int(g["steps"])):
        rom.advance(x, float(g["dt"]), 1, gn_iters=int(g["updates"]), tol=0.0, order=int(g["order"]),
                    first_step=n + 1)
        got = x.cpu().numpy()
        assert np.allclose(got, g["traj"][n], rtol=1e-8, atol=1e-10 * scale), (n, got, g["traj"][n])
