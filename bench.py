#!/usr/bin/env python3
"""Benchmark: FP64 finite-volume residual ("velocity") throughput.

Workload (default): 2D Euler four-quadrant Riemann problem (IC2), 1024x1024
cells on [0,1]^2, WENO5 + Rusanov, FP64, state = IC + seeded U[-1e-3, 1e-3]
noise, transmissive (Neumann) boundaries; one step = one velocity()
evaluation of the whole mesh.  value = Gcell/s with the state resident in
HBM; e2e = the same metric through the host-buffer C-ABI call
(pda_velocity_host: H2D state copy, kernels, D2H velocity copy per step).

--impl reference times the reference's CPU algorithm for the same workload
on all host cores (the oracle restatement; the reference C++ itself is not
compiled on the GPU host).  Under torchrun with N>1 each rank runs an
independent replica (the path does not shard); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_CELLS_SIDE = 1024
NDPC = 4
BYTES_PER_CELL = 16 * NDPC  # read U once + write V once (FP64)
# Algorithmic FP64 operations per cell of the face-once WENO5 + Rusanov 2D
# Euler velocity (counted from the kernel source: per face 4 x 2 one-sided
# WENO5 values at 71 flops + 4 divisions each, one Rusanov flux at 65 flops
# + 10 divisions + 3 square roots; two faces per cell plus the 24-flop
# balance; a division or square root counts as one operation).
# DRAM bytes (read + write) per cell of one face launch, measured by ncu on
# k_faces_tile at 2048^2 (x-axis launch: 135.3 MB read + 96.3 MB written);
# traffic grows in proportion to the cells, so it scales to other sizes
FACE_TRAFFIC_BYTES_PER_CELL = (135.32e6 + 96.27e6) / 2048 ** 2
# FP64 instructions the face kernel executes per face (ncu thread-instruction
# counters dadd + dmul + dfma of the same capture, 270.7 per face): the work
# the FP64 pipe actually does, after the divisions, square roots and
# products by constants moved to the integer pipe
FP64_INST_PER_FACE = 270.7
FLOPS_PER_CELL = 2 * (4 * 2 * (71 + 4) + 65 + 10 + 3) + 24
L2_FLUSH_BYTES = 256 << 20


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region: one query every 20 ms,
    started (first sample received) before the region begins."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.005)
            self.lines.clear()  # the region starts now: drop the sample taken before it
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(pda, torch, stream):
    mesh = pda.create_full_mesh((N_CELLS_SIDE, N_CELLS_SIDE), (0.0, 1.0, 0.0, 1.0), 7)
    prob = pda.create_problem(mesh, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2, stream=stream)
    U0 = prob.initialConditionHost()
    rng = np.random.default_rng(20261203)
    U = U0 + rng.uniform(-1e-3, 1e-3, U0.shape)
    return mesh, prob, U


def oracle_workload(threads=0):
    """The headline workload built by the oracle alone: the mesh from
    oracle/mesh_gen.py (the reference's mesh-script layout), the initial
    condition from the oracle's restatement of riemann2dIC2 and the same
    seeded noise; nothing from the library."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import mesh_gen
    import oracle_py
    orc = oracle_py.load()
    used = orc.set_threads(threads if threads > 0 else (os.cpu_count() or 1))
    mg = mesh_gen.full_mesh((N_CELLS_SIDE, N_CELLS_SIDE), (0.0, 1.0, 0.0, 1.0), 7, orc=orc)
    op = orc.problem(mg.oracle_mesh(orc), 1, 4, 2, 2)
    U0 = op.initial_condition()
    rng = np.random.default_rng(20261203)
    return orc, op, U0 + rng.uniform(-1e-3, 1e-3, U0.shape), used


def cpu_baseline(U, V_gpu, budget_s=10.0, threads=0):
    """The oracle (C restatement of the reference algorithm) on the host
    cores: all threads for the reported value, one thread beside it, and the
    oracle's velocity compared with the GPU's (the line's parity field)."""
    orc, op, Uo, used = oracle_workload(threads)
    assert np.array_equal(U, Uo), "the library's and the oracle's workloads differ"
    Vo = op.velocity(U)  # warm-up, and the parity reference
    times = []
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end or len(times) < 2:
        t0 = time.perf_counter()
        op.velocity(U)
        times.append(time.perf_counter() - t0)
    cells = N_CELLS_SIDE * N_CELLS_SIDE
    med = statistics.median(times)
    orc.set_threads(1)
    t0 = time.perf_counter()
    op.velocity(U)
    one = time.perf_counter() - t0
    orc.set_threads(used)
    import platform
    diff = np.abs(V_gpu - Vo)
    scale = np.maximum(np.abs(Vo), 1e-3 * np.max(np.abs(Vo.reshape(-1, NDPC)), axis=0)[None, :].repeat(
        Vo.size // NDPC, axis=0).reshape(-1))
    parity = {"reference": "oracle (C restatement, bit-identical to the reference on the golden cases)",
              "bitwise": bool(np.array_equal(V_gpu, Vo)), "max_abs": float(diff.max()),
              "max_rel": float(np.max(diff / scale)), "rule": "per cell, floor 1e-3 x field max"}
    base = {"value": cells / med / 1e9, "unit": "Gcell/s", "cores": used, "kind": "port",
            "sample": f"{len(times)} velocity() calls of the same 1024^2 Riemann WENO5 workload on {used} "
                      f"threads of {platform.machine()} ({os.cpu_count()} logical CPUs); median "
                      f"{med * 1e3:.1f} ms/call",
            "single_thread": {"value": cells / one / 1e9, "unit": "Gcell/s", "cores": 1,
                              "sample": f"one call on 1 thread, {one * 1e3:.0f} ms"}}
    return base, parity


def run_reference(args):
    """The reference's CPU algorithm (the oracle port; the reference C++ is
    header-only and not on the GPU host) on all host cores, mesh and initial
    condition from the oracle itself: no library code on this path."""
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    orc, op, U, used = oracle_workload()
    for _ in range(args.warmup):
        op.velocity(U)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        op.velocity(U)
        ts.append(time.perf_counter() - t0)
    ms = 1e3 * sum(ts) / len(ts)
    cells = N_CELLS_SIDE * N_CELLS_SIDE
    value = cells / (ms * 1e-3) / 1e9
    import platform
    line = {"impl": "reference", "metric": "FV residual Gcell/s", "value": value, "unit": "Gcell/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (Riemann IC2 + seeded U[-1e-3,1e-3] noise)",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "Gcell/s", "cores": used, "kind": "port",
                             "sample": f"{args.steps} full 1024^2 velocity() calls on {used} threads of "
                                       f"{platform.machine()}; the oracle's C restatement, bit-identical to "
                                       f"the reference (header-only C++, no checkout on the GPU host); mesh "
                                       f"and initial condition built by the oracle"},
            "e2e": {"value": value, "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _time_gpu(torch, stream, fn, reps, warm=2):
    for _ in range(warm):
        fn()
    stream.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    with torch.cuda.stream(stream):
        for a, b in ev:
            a.record(stream)
            fn()
            b.record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / reps


def _cpu_rate(fn, budget_s):
    fn()
    ts = []
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end or not ts:
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts), len(ts)


class _Ctx:
    """What every secondary workload needs: the package, torch, the stream,
    the oracle (None without CPU baselines) and its thread count."""

    def __init__(self, pda, torch, stream, cpu):
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle_py
        self.pda, self.torch, self.stream = pda, torch, stream
        self.orc = oracle_py.load() if cpu else None
        self.threads = self.orc.set_threads(os.cpu_count() or 1) if cpu else 0
        self.rng = np.random.default_rng(20261203)

    def oracle_problem(self, mesh, fam, prob, scheme, ic, dim, st):
        g, x, y, z, _, _ = mesh._arrays()
        om = self.orc.mesh_from_arrays(dim, st, g, x, y, z, (mesh.dx(), mesh.dy(), mesh.dz()))
        return om, self.orc.problem(om, fam, prob, scheme, ic)


def wl_jacobian_2d(c):
    """2D Euler Riemann WENO5 Jacobian (V + CSR J), 1024^2 (PDA_JAC_N overrides
    the size for profiling runs)"""
    pda, torch, stream, orc, threads, rng = c.pda, c.torch, c.stream, c.orc, c.threads, c.rng
    cpu = orc is not None
    oracle_problem = c.oracle_problem
    n = int(os.environ.get("PDA_JAC_N", 1024))
    mesh = pda.create_full_mesh((n, n), (0.0, 1.0, 0.0, 1.0), 7)
    prob = pda.create_problem(mesh, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2, stream=stream)
    Uh = prob.initialConditionHost() + rng.uniform(-1e-3, 1e-3, 4 * n * n)
    with torch.cuda.stream(stream):
        U = torch.from_numpy(Uh).cuda()
        V = prob.createVelocity()
        J = prob.createJacobian()
    ms = _time_gpu(torch, stream, lambda: prob.rightHandSideAndJacobian(U, 0.0, V, J), 5)
    nnz = J.nonZeros()
    with torch.cuda.stream(stream):
        U.copy_(torch.from_numpy(prob.initialConditionHost()))
    ms_ic = _time_gpu(torch, stream, lambda: prob.rightHandSideAndJacobian(U, 0.0, V, J), 5)
    w = {"config": f"euler2d_riemann_ic2_weno5_jacobian_{n}x{n}", "ms_per_call": ms, "nnz": nnz,
         "value": nnz / (ms * 1e-3) / 1e9, "unit": "Gnnz/s (V + CSR J per call)",
         "gcell_per_s": n * n / (ms * 1e-3) / 1e9,
         "on_initial_condition": {"ms_per_call": ms_ic, "value": nnz / (ms_ic * 1e-3) / 1e9}}
    del U, V, J, prob
    torch.cuda.empty_cache()
    if cpu:
        ns = 256
        m2 = pda.create_full_mesh((ns, ns), (0.0, 1.0, 0.0, 1.0), 7)
        p2 = pda.create_problem(m2, pda.Euler2d.Riemann, pda.InviscidFluxReconstruction.Weno5, 2, stream=0)
        U2 = p2.initialConditionHost() + rng.uniform(-1e-3, 1e-3, 4 * ns * ns)
        om, op = oracle_problem(m2, 1, 4, 2, 2, 2, 7)
        med, k = _cpu_rate(lambda: op.velocity_and_jacobian(U2), 5.0)
        w["cpu_baseline"] = {"value": op.nnz / med / 1e9, "unit": "Gnnz/s", "cores": threads, "kind": "port",
                             "sample": f"{k} V+J calls at 256^2 (same problem/scheme), median {med*1e3:.1f} ms"}
        U2ic = p2.initialConditionHost()
        med, k = _cpu_rate(lambda: op.velocity_and_jacobian(U2ic), 2.0)
        w["cpu_baseline"]["on_initial_condition"] = {"value": op.nnz / med / 1e9, "sample": f"{k} calls at 256^2"}
    return w


def wl_jacobian_swe(c, n=1024, ns=256):
    """2D shallow water, slip walls, WENO5, V + CSR J at 1024^2 (the reference's
    default parameters: gravity 9.8, Coriolis -3, pulse 0.125).  The CPU leg
    runs one thread: the reference's threaded near-boundary Jacobian loop of
    this problem races on a shared member, so its J is timed serially."""
    pda, torch, stream, orc, rng = c.pda, c.torch, c.stream, c.orc, c.rng
    params = {"gravity": 9.8, "coriolis": -3.0, "pulseMagnitude": 0.125}
    mesh = pda.create_full_mesh((n, n), (-5.0, 5.0, -5.0, 5.0), 7)
    prob = pda.create_problem(mesh, pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 1, params,
                              stream=stream)
    Uh = prob.initialConditionHost() + rng.uniform(-1e-3, 1e-3, 3 * n * n)
    with torch.cuda.stream(stream):
        U = torch.from_numpy(Uh).cuda()
        V = prob.createVelocity()
        J = prob.createJacobian()
    ms = _time_gpu(torch, stream, lambda: prob.rightHandSideAndJacobian(U, 0.0, V, J), 5)
    nnz = J.nonZeros()
    w = {"config": f"swe2d_slipwall_weno5_jacobian_{n}x{n}", "ms_per_call": ms, "nnz": nnz,
         "value": nnz / (ms * 1e-3) / 1e9, "unit": "Gnnz/s (V + CSR J per call)"}
    del U, V, J, prob
    torch.cuda.empty_cache()
    if orc is not None:
        m2 = pda.create_full_mesh((ns, ns), (-5.0, 5.0, -5.0, 5.0), 7)
        g, x, y, z, _, _ = m2._arrays()
        om = orc.mesh_from_arrays(2, 7, g, x, y, z, (m2.dx(), m2.dy(), m2.dz()))
        op = orc.problem(om, 3, 0, 2, 1, params)
        U2 = op.initial_condition() + rng.uniform(-1e-3, 1e-3, 3 * ns * ns)
        used = orc.set_threads(1)
        med, k = _cpu_rate(lambda: op.velocity_and_jacobian(U2), 3.0)
        orc.set_threads(c.threads)
        w["cpu_baseline"] = {"value": op.nnz / med / 1e9, "unit": "Gnnz/s", "cores": used, "kind": "port",
                             "sample": f"{k} V+J calls at {ns}^2 on 1 thread, median {med*1e3:.0f} ms"}
    return w


def wl_velocity_3d(c):
    """3D Euler smooth periodic WENO5 velocity, 256^3"""
    pda, torch, stream, orc, threads, rng = c.pda, c.torch, c.stream, c.orc, c.threads, c.rng
    cpu = orc is not None
    oracle_problem = c.oracle_problem
    n = 256
    mesh = pda.create_full_mesh((n, n, n), (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 7, (True, True, True))
    prob = pda.create_problem(mesh, pda.Euler3d.PeriodicSmooth, pda.InviscidFluxReconstruction.Weno5, stream=stream)
    with torch.cuda.stream(stream):
        U = prob.initialCondition()
        V = prob.createVelocity()
    ms = _time_gpu(torch, stream, lambda: prob.velocity(U, 0.0, V), 5)
    prof = prob.profile_velocity(U, V, reps=3)
    w = {"config": "euler3d_smooth_periodic_weno5_velocity_256^3", "ms_per_call": ms,
         "value": n ** 3 / (ms * 1e-3) / 1e9, "unit": "Gcell/s", "kernel_ms": prof}
    # WENO3, the reference's own 3D scheme (its 3D path has no WENO5)
    p3 = pda.create_problem(mesh, pda.Euler3d.PeriodicSmooth, pda.InviscidFluxReconstruction.Weno3, stream=stream)
    ms3 = _time_gpu(torch, stream, lambda: p3.velocity(U, 0.0, V), 5)
    w["weno3"] = {"ms_per_call": ms3, "value": n ** 3 / (ms3 * 1e-3) / 1e9, "unit": "Gcell/s"}
    del U, V, prob, p3
    torch.cuda.empty_cache()
    if cpu:
        ns = 64
        m3 = pda.create_full_mesh((ns, ns, ns), (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 7, (True, True, True))
        om, op = oracle_problem(m3, 2, 0, 2, 1, 3, 7)
        U3 = op.initial_condition()
        med, k = _cpu_rate(lambda: op.velocity(U3), 5.0)
        w["cpu_baseline"] = {"value": ns ** 3 / med / 1e9, "unit": "Gcell/s", "cores": threads, "kind": "port",
                             "sample": f"{k} velocity calls at 64^3 (same problem/scheme), median {med*1e3:.1f} ms"}
        om3, op3 = oracle_problem(m3, 2, 0, 1, 1, 3, 7)
        med, k = _cpu_rate(lambda: op3.velocity(U3), 2.0)
        w["weno3"]["cpu_baseline"] = {"value": ns ** 3 / med / 1e9, "unit": "Gcell/s", "cores": threads,
                                      "kind": "port", "sample": f"{k} WENO3 velocity calls at 64^3"}
    return w


def wl_jacobian_3d(c):
    """3D Euler WENO5 Jacobian, 96^3 (PDA_JAC3_N overrides the size for
    profiling runs)"""
    pda, torch, stream, orc, threads, rng = c.pda, c.torch, c.stream, c.orc, c.threads, c.rng
    cpu = orc is not None
    oracle_problem = c.oracle_problem
    n = int(os.environ.get("PDA_JAC3_N", 96))
    mesh = pda.create_full_mesh((n, n, n), (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 7, (True, True, True))
    prob = pda.create_problem(mesh, pda.Euler3d.PeriodicSmooth, pda.InviscidFluxReconstruction.Weno5, stream=stream)
    with torch.cuda.stream(stream):
        U = prob.initialCondition()
        V = prob.createVelocity()
        J = prob.createJacobian()
    ms = _time_gpu(torch, stream, lambda: prob.rightHandSideAndJacobian(U, 0.0, V, J), 3)
    nnz = J.nonZeros()
    w = {"config": f"euler3d_smooth_periodic_weno5_jacobian_{n}^3", "ms_per_call": ms, "nnz": nnz,
         "value": nnz / (ms * 1e-3) / 1e9, "unit": "Gnnz/s (V + CSR J per call)"}
    del U, V, J, prob
    torch.cuda.empty_cache()
    if cpu:
        ns = 24
        m3 = pda.create_full_mesh((ns, ns, ns), (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 7, (True, True, True))
        om, op = oracle_problem(m3, 2, 0, 2, 1, 3, 7)
        U3 = op.initial_condition()
        med, k = _cpu_rate(lambda: op.velocity_and_jacobian(U3), 5.0)
        w["cpu_baseline"] = {"value": op.nnz / med / 1e9, "unit": "Gnnz/s", "cores": threads, "kind": "port",
                             "sample": f"{k} V+J calls at 24^3 (same problem/scheme), median {med*1e3:.1f} ms"}
    return w


def wl_sod_1d_ssprk3(c):
    """1D Sod, WENO5, SSP-RK3 dt=1e-4, 2000 steps (CUDA-graph steps)"""
    pda, torch, stream, orc, threads, rng = c.pda, c.torch, c.stream, c.orc, c.threads, c.rng
    cpu = orc is not None
    oracle_problem = c.oracle_problem
    mesh = pda.create_full_mesh((1000,), (-0.5, 0.5), 7)
    prob = pda.create_problem(mesh, pda.Euler1d.Sod, pda.InviscidFluxReconstruction.Weno5, stream=stream)
    with torch.cuda.stream(stream):
        U = prob.initialCondition()
    prob.advance_ssprk3(U, 0.0, 1e-4, 10)  # capture + warm-up
    stream.synchronize()
    with torch.cuda.stream(stream):
        U = prob.initialCondition()
    stream.synchronize()
    t0 = time.perf_counter()
    prob.advance_ssprk3(U, 0.0, 1e-4, 2000)
    stream.synchronize()
    wall = time.perf_counter() - t0
    w = {"config": "euler1d_sod_weno5_ssprk3_dt1e-4_2000_steps_1000_cells", "wall_ms": wall * 1e3,
         "value": 3 * 2000 * 1000 / wall / 1e9, "unit": "Gcell-updates/s",
         "note": "whole run timed on the host clock, steps replayed from a CUDA graph"}
    if cpu:
        om, op = oracle_problem(mesh, 0, 1, 2, 1, 1, 7)
        orc.set_threads(1)
        Uo = op.initial_condition()
        t0 = time.perf_counter()
        op.ssprk3(Uo, 0.0, 1e-4, 2000)
        cw = time.perf_counter() - t0
        orc.set_threads(os.cpu_count() or 1)
        w["cpu_baseline"] = {"value": 3 * 2000 * 1000 / cw / 1e9, "unit": "Gcell-updates/s", "cores": 1,
                             "kind": "port", "sample": f"the full 2000-step run, 1 thread, {cw*1e3:.0f} ms"}
        w["final_state_matches_oracle"] = bool(np.allclose(U.cpu().numpy(), Uo, rtol=1e-12, atol=1e-13))
    return w


def wl_ssprk3_3d(c):
    """3D Euler smooth periodic WENO5, SSP-RK3 at CFL 0.4, 256^3 (a few of the 200 steps)"""
    pda, torch, stream, orc, threads, rng = c.pda, c.torch, c.stream, c.orc, c.threads, c.rng
    cpu = orc is not None
    oracle_problem = c.oracle_problem
    n = 256
    mesh = pda.create_full_mesh((n, n, n), (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 7, (True, True, True))
    prob = pda.create_problem(mesh, pda.Euler3d.PeriodicSmooth, pda.InviscidFluxReconstruction.Weno5, stream=stream)
    # max over cells of |u_axis| + c on the IC (u = 1, p = 1, rho >= 0.8)
    dt = 0.4 * (2.0 / n) / (1.0 + (1.4 * 1.0 / 0.8) ** 0.5)
    with torch.cuda.stream(stream):
        U = prob.initialCondition()
    prob.advance_ssprk3(U, 0.0, dt, 1)  # capture + warm-up
    k3 = 2
    ms = _time_gpu(torch, stream, lambda: prob.advance_ssprk3(U, 0.0, dt, k3), 1, warm=0)
    w = {"config": "euler3d_smooth_periodic_weno5_ssprk3_cfl0.4_256^3", "dt": dt, "steps_timed": k3,
         "ms_per_step": ms / k3, "value": 3 * n ** 3 * k3 / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s",
         "projected_200_steps_s": 200 * ms / k3 * 1e-3}
    del U, prob
    torch.cuda.empty_cache()
    if cpu:
        ns = 64
        m3 = pda.create_full_mesh((ns, ns, ns), (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0), 7, (True, True, True))
        om, op = oracle_problem(m3, 2, 0, 2, 1, 3, 7)
        U3 = op.initial_condition()
        med, k = _cpu_rate(lambda: op.ssprk3(U3, 0.0, dt, 1), 5.0)
        w["cpu_baseline"] = {"value": 3 * ns ** 3 / med / 1e9, "unit": "Gcell-updates/s", "cores": threads,
                             "kind": "port", "sample": f"{k} SSP-RK3 steps at 64^3, median {med*1e3:.1f} ms"}
    return w


def wl_batched_swe(c):
    return batched_swe_workload(c.pda, c.torch, c.stream, c.orc, c.threads)


def _pkg_module(name):
    import importlib.util
    spec = importlib.util.spec_from_file_location("pda_gb300_" + name,
                                                  os.path.join(REPO, "pressio-demoapps_gb300", name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rom_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("pda_gb300_rom", os.path.join(REPO, "pressio-demoapps_gb300",
                                                                                 "rom.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def wl_rom_swe(c, n=256, n_train=48, n_snap=400, n_test=8, latent=12, epochs=int(os.environ.get("PDA_ROM_EPOCHS", 150)),
               batch=128, lr=1e-3, dt=0.005, rom_ratio=int(os.environ.get("PDA_ROM_RATIO", 5)), gn_iters=1,
               order=int(os.environ.get("PDA_ROM_ORDER", 2))):
    """Learned-manifold hyper-reduced LSPG on 2D SWE slip wall 256^2: 48
    Latin-hypercube training points (gravity, coriolis, pulse), 400 FOM
    snapshots each (SSP-RK3 dt 0.005, batched device FOM), MLP autoencoder
    latent 12, hidden 256 / 1024, ELU, full-width output, trained on the device
    (BF16 tcgen05 GEMMs, fp32 accumulation, Adam); sample mesh 1 % of the cells
    (fixed seed) + WENO5 stencils; LSPG with BDF2 (first step BDF1) and
    Gauss-Newton (FP64 normal equations) on 8 held-out points, the FOM as the
    fallback whenever a stretch's Gauss-Newton residual exceeds a threshold;
    wall time and relative L2 error against the single-point GPU FOM, and the
    same for POD-LSPG with the same latent size (the method without the
    learned part)."""
    R = _rom_module()
    pda, torch = c.pda, c.torch
    out = {"config": f"swe_slipwall_256^2_weno5_learned_lspg_bdf{order}_latent12", "train_points": n_train,
           "snapshots_per_point": n_snap, "test_points": n_test, "latent": latent, "epochs": epochs,
           "dt_fom": dt, "dt_rom": dt * rom_ratio, "gn_iters_max": gn_iters, "bdf_order": order,
           "gauss_newton": "residual, normal equations and solve fp64; Jacobian terms fp32 (inexact step)"}
    setup = R.SweSetup(pda, n)
    train = R.latin_hypercube(n_train, seed=5)
    test = R.uniform_points(n_test, seed=6)
    t0 = time.perf_counter()
    S = setup.snapshots(train, dt, n_snap)
    torch.cuda.synchronize()
    out["snapshots_s"] = time.perf_counter() - t0
    scale = setup.normalization(S)
    X = setup.training_data(S, scale)
    phi = R.pod_basis(S, setup.uref, latent)
    del S
    torch.cuda.empty_cache()
    ae = pda.AutoEncoder(setup.N, latent, 1024, 256, seed=1, stream=setup.stream)
    t0 = time.perf_counter()
    losses = R.train_schedule(ae, X, epochs, batch=batch, lr=lr, seed=2)
    out["train_s"] = time.perf_counter() - t0
    out["loss_first_last"] = [float(losses[0]), float(losses[-1])]
    del X
    torch.cuda.empty_cache()
    learned = R.LearnedRom(setup, ae, scale)
    sm, gids, st, s2st = setup.sample_mesh(0.01, seed=7)
    out["sample_cells"], out["stencil_cells"] = int(len(gids)), int(len(st))
    fdec, _fp = learned.full_decoder()
    fp_aff = setup.problem({"gravity": 9.8, "coriolis": -3.0, "pulseMagnitude": 0.125})
    faff = pda.LspgRom.affine(fp_aff, np.arange(n * n), setup.uref, phi)
    checkpoints = [100, 200, 300, 400]

    def make_rom(p, kind, sample=(sm, st, s2st)):
        smesh, stc, s2 = sample
        ps = setup.problem(p, mesh=smesh)
        U0 = setup.problem(p).initialCondition()
        if kind == "learned":
            return learned.lspg(ps, s2, stc, tensor_cores=True), learned.encode(U0), fdec
        return R.affine_lspg(setup, phi, ps, s2, stc), (phi.T @ (U0 - setup.uref)).contiguous(), faff

    def run_point(p, kind, threshold, gn=gn_iters, ratio=rom_ratio, ordr=order, sample=(sm, st, s2st)):
        rom, x0, dec = make_rom(p, kind, sample)
        return R.FallbackRun(setup, p, rom, dec, x0, dt, ratio, checkpoints, threshold, gn_iters=gn, order=ordr)

    # residual threshold for the FOM fallback: 5x the largest Gauss-Newton
    # residual norm seen over a training point's trajectory
    rom0, x00, _ = make_rom(train[0], "learned")
    _, _, res_train = R.run_rom(rom0, x00, dt * rom_ratio, [cp // rom_ratio for cp in checkpoints], setup.stream,
                                gn_iters=gn_iters, order=order)
    threshold = 5.0 * res_train
    out["fallback_residual_threshold"] = threshold
    pts = []
    for p in test:
        states, fom_wall = setup.fom_trajectory(p, dt, checkpoints)
        rec = {"params": p, "fom_s": fom_wall}
        # best the trial manifold can do: decoder(encoder(FOM state)), and the POD projection
        rec["learned_projection_rel_l2"] = [R.rel_l2(fdec.decode(learned.encode(states[cp])), states[cp])
                                            for cp in checkpoints]
        rec["pod_projection_rel_l2"] = [R.rel_l2(setup.uref + phi @ (phi.T @ (states[cp] - setup.uref)), states[cp])
                                        for cp in checkpoints]
        for kind in ("learned", "pod"):
            run = run_point(p, kind, threshold if kind == "learned" else float("inf"))
            errs = [R.rel_l2(run.states[cp], states[cp]) for cp in checkpoints]
            errp = [R.rel_l2(run.states[cp], states[cp], setup.uref) for cp in checkpoints]
            rec[kind] = {"rom_s": run.wall, "speedup": fom_wall / run.wall, "rel_l2_state": errs,
                         "rel_l2_perturbation": errp, "fallback_at_step": run.fallback_at}
        pts.append(rec)
    out["points"] = pts
    L = [q["learned"] for q in pts]
    P = [q["pod"] for q in pts]
    fom = [q["fom_s"] for q in pts]
    out["summary"] = {
        "fom_s_per_point": float(np.mean(fom)),
        "rom_s_per_point": float(np.mean([q["rom_s"] for q in L])),
        "rom_s_per_point_median": float(np.median([q["rom_s"] for q in L])),
        "rom_s_points": [float(q["rom_s"]) for q in L],
        "speedup": float(np.sum(fom) / np.sum([q["rom_s"] for q in L])),
        "speedup_median": float(np.median([q["speedup"] for q in L])),
        "rel_l2_state_final_mean": float(np.mean([q["rel_l2_state"][-1] for q in L])),
        "rel_l2_state_max": float(np.max([max(q["rel_l2_state"]) for q in L])),
        "rel_l2_perturbation_final_mean": float(np.mean([q["rel_l2_perturbation"][-1] for q in L])),
        "pod_rel_l2_state_final_mean": float(np.mean([q["rel_l2_state"][-1] for q in P])),
        "pod_rel_l2_state_max": float(np.max([max(q["rel_l2_state"]) for q in P])),
        "pod_rel_l2_perturbation_final_mean": float(np.mean([q["rel_l2_perturbation"][-1] for q in P])),
        "pod_speedup": float(np.sum(fom) / np.sum([q["rom_s"] for q in P])),
        "fallbacks": int(sum(q["fallback_at_step"] is not None for q in L)),
        "learned_projection_rel_l2_final_mean": float(np.mean([q["learned_projection_rel_l2"][-1] for q in pts])),
        "pod_projection_rel_l2_final_mean": float(np.mean([q["pod_projection_rel_l2"][-1] for q in pts])),
    }
    # further (order : Gauss-Newton iterations : ROM step / FOM step [: sample
    # fraction]) settings of the same trained network: the speed / accuracy
    # trade-off of the step and of the sample mesh
    variants = [v for v in os.environ.get("PDA_ROM_VARIANTS", "1:1:5,2:1:2,2:1:4,2:2:5,2:1:10,2:1:5:0.03").split(",")
                if v]
    if variants:
        out["variants"] = {}
        states_by_point = [setup.fom_trajectory(p, dt, checkpoints) for p in test]
        for v in variants:
            f = v.split(":")
            ordr, gn, ratio = (int(u) for u in f[:3])
            frac = float(f[3]) if len(f) > 3 else 0.01
            if any(cp % ratio for cp in checkpoints):
                out["variants"][v] = {"skipped": f"checkpoints {checkpoints} are not multiples of {ratio}"}
                continue
            if frac != 0.01:
                sm_v, gids_v, st_v, s2st_v = setup.sample_mesh(frac, seed=7)
                sample = (sm_v, st_v, s2st_v)
            else:
                sample = (sm, st, s2st)
            walls, fwalls, errs = [], [], []
            for p, (states, fw) in zip(test, states_by_point):
                run = run_point(p, "learned", float("inf"), gn, ratio, ordr, sample)
                walls.append(run.wall)
                fwalls.append(fw)
                errs.append(max(R.rel_l2(run.states[cp], states[cp]) for cp in checkpoints))
            out["variants"][v] = {"bdf_order": ordr, "gn_iters": gn, "dt_rom": dt * ratio, "sample_fraction": frac,
                                  "sample_cells": int(len(sample[2])),
                                  "speedup": float(sum(fwalls) / sum(walls)),
                                  "rel_l2_state_max": float(max(errs)), "rel_l2_state_mean_of_max": float(np.mean(errs))}
    if c.orc is not None:
        # the FOM on the host cores (oracle), one point, a bounded number of steps
        import tempfile
        d = tempfile.mkdtemp()
        setup.mesh.write(d)
        om = c.orc.mesh_load(d)
        op = c.orc.problem(om, 3, 0, 2, 1, test[0])
        Uo = op.initial_condition()
        t0 = time.perf_counter()
        op.ssprk3(Uo, 0.0, dt, 20)
        cw = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": cw / 20 * n_snap, "unit": "s per FOM trajectory (400 steps)",
                               "cores": c.threads, "kind": "port",
                               "sample": f"20 SSP-RK3 steps of one test point on the host, {cw:.2f} s, x20"}
    del ae, learned, fdec, faff
    torch.cuda.empty_cache()
    return out


def wl_lspg_step(c, n=256, latent=12, steps=20, gn_iters=3):
    """Latency of one hyper-reduced LSPG step (BDF1, Gauss-Newton, CUDA-graph
    replay) on the 1 % sample mesh of the 256^2 shallow-water problem, with an
    affine basis and with an MLP decoder of the config-5 shape (random weights,
    no training: the step's cost does not depend on the weights' values)."""
    R = _rom_module()
    pda, torch = c.pda, c.torch
    setup = R.SweSetup(pda, n)
    sm, gids, st, s2st = setup.sample_mesh(0.01, seed=7)
    ps = setup.problem({"gravity": 7.0, "coriolis": -2.0, "pulseMagnitude": 0.1}, mesh=sm)
    g = torch.Generator(device="cuda").manual_seed(0)
    phi = torch.randn(setup.N, latent, generator=g, device="cuda", dtype=torch.float64) * (0.3 / setup.N ** 0.5)
    W1 = torch.randn(256, latent, generator=g, device="cuda") * 0.3
    b1 = torch.randn(256, generator=g, device="cuda") * 0.1
    W2 = torch.randn(1024, 256, generator=g, device="cuda") * 0.05
    b2 = torch.randn(1024, generator=g, device="cuda") * 0.1
    W3 = torch.randn(setup.N, 1024, generator=g, device="cuda") * 0.02
    b3 = torch.randn(setup.N, generator=g, device="cuda") * 0.1
    scale = torch.full((setup.N,), 0.05, dtype=torch.float64, device="cuda")
    learned = R.LearnedRom.__new__(R.LearnedRom)
    learned.setup, learned.scale, learned.dec = setup, scale, (W1, b1, W2, b2, W3, b3)
    out = {"config": "lspg_bdf1_swe256_sample1pct", "sample_cells": int(len(gids)), "stencil_cells": int(len(st)),
           "gn_iters": gn_iters, "steps_timed": steps}
    learned.dec = tuple(t.to(torch.bfloat16).float() if t.dim() == 2 else t for t in learned.dec)
    # the first three with the exact (double) Jacobian, the last two with its
    # terms in single precision (the ROM's default: an inexact Gauss-Newton step)
    for kind, rom in (("affine", R.affine_lspg(setup, phi, ps, s2st, st, jacobian_bits=64)),
                      ("mlp_fp32", learned.lspg(ps, s2st, st, tensor_cores=False, jacobian_bits=64)),
                      ("mlp_tensor_cores", learned.lspg(ps, s2st, st, tensor_cores=True, jacobian_bits=64)),
                      ("affine_jac32", R.affine_lspg(setup, phi, ps, s2st, st, jacobian_bits=32)),
                      ("mlp_tensor_cores_jac32", learned.lspg(ps, s2st, st, tensor_cores=True, jacobian_bits=32))):
        x = torch.zeros(latent, dtype=torch.float64, device="cuda")
        rom.advance_bdf1(x, 0.02, 2, gn_iters, 0.0)  # capture + warm-up; tol 0: every iteration runs
        setup.stream.synchronize()
        t0 = time.perf_counter()
        rom.advance_bdf1(x, 0.02, steps, gn_iters, 0.0)
        setup.stream.synchronize()
        wall = time.perf_counter() - t0
        out[kind] = {"ms_per_step": 1e3 * wall / steps, "ms_per_gn_iteration": 1e3 * wall / steps / gn_iters}
    return out


def wl_ae_step(c, n=3 * 256 * 256, latent=12, ha=1024, hb=256, batch=128, steps=24):
    """One Adam step of the ROM's autoencoder (n = 196,608 outputs = 256^2
    shallow-water cells x 3, latent 12, hidden 1024 / 256, batch 128) on seeded
    random bf16 rows: forward and backward tcgen05 GEMMs, ELU, squared error,
    Adam; with Adam fused into the weight-gradient GEMMs (the library's
    default) and as a separate pass.  HBM floor of a step: every weight once
    through the schedule -- bf16 copy read by the forward GEMM (2 B), fp32
    weight and moments read and written (24 B), bf16 copy written (2 B), and
    for the layers whose input gradient is needed the bf16 transpose read and
    written (4 B): 28 or 32 B per weight."""
    pda, torch = c.pda, c.torch
    n = int(os.environ.get("PDA_AE_N", n))  # smaller outputs for profiling captures
    steps = int(os.environ.get("PDA_AE_STEPS", steps))
    g = torch.Generator(device="cuda").manual_seed(0)
    X = (torch.rand(batch * steps, n, generator=g, device="cuda") * 2 - 1).to(torch.bfloat16)
    shapes = list(zip((n, ha, hb, latent, hb, ha), (ha, hb, latent, hb, ha, n)))
    params = sum(i * o + o for i, o in shapes)
    floor_bytes = sum(i * o * (28 if l == 0 else 32) for l, (i, o) in enumerate(shapes))
    hbm, src = measured_peaks()
    floor_ms = floor_bytes / (hbm * 1e9) * 1e3
    out = {"config": f"autoencoder_adam_step_n{n}_latent12_hidden1024_256_batch128", "parameters": params,
           "hbm_floor_bytes_per_step": floor_bytes, "hbm_floor_ms": floor_ms, "peak_source": src,
           "note": "host clock around whole epochs of the library's training loop (one loss read back per step)"}
    for fused in (True, False):
        ae = pda.AutoEncoder(n, latent, ha, hb, seed=1, stream=c.stream)
        ae.set_fused(fused)
        ae.train(X[: batch * 4], batch=batch, epochs=1, lr=1e-3, seed=0)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ae.train(X, batch=batch, epochs=1, lr=1e-3, seed=1)
        torch.cuda.synchronize()
        ms = 1e3 * (time.perf_counter() - t0) / steps
        out["fused_adam" if fused else "separate_adam"] = {"ms_per_step": ms, "hbm_floor_fraction": floor_ms / ms}
        del ae
    del X
    return out


# workloads whose work is split over the ranks (every rank must run them)
SHARDED = {"batched_swe"}

WORKLOADS = {"jacobian_2d": wl_jacobian_2d, "jacobian_swe": wl_jacobian_swe, "velocity_3d": wl_velocity_3d,
             "jacobian_3d": wl_jacobian_3d,
             "sod_1d_ssprk3": wl_sod_1d_ssprk3, "ssprk3_3d": wl_ssprk3_3d, "batched_swe": wl_batched_swe,
             "rom_swe": wl_rom_swe, "lspg_step": wl_lspg_step, "ae_step": wl_ae_step}


def extra_workloads(pda, torch, stream, cpu=True, names=None):
    """Secondary configurations, one JSON object each (default: all)."""
    c = _Ctx(pda, torch, stream, cpu)
    out = {}
    for name in (list(WORKLOADS) if names is None else names):
        out[name] = WORKLOADS[name](c)
        torch.cuda.empty_cache()
    return out


def batched_swe_workload(pda, torch, stream, orc, threads, n_inst=512, steps=3):
    """512 shallow-water slip-wall instances on [-5,5]^2, n drawn seeded from
    {64, 96, ..., 512}, gravity ~ U[5,10], coriolis ~ U[-4,-1], pulse
    magnitude ~ U[0.05,0.2]; WENO5, SSP-RK3 dt = 0.005.  Times a few of the
    500 steps of the whole batch (one CUDA graph per step), the same steps
    launched instance by instance, and the oracle on a sample of instances."""
    brng = np.random.default_rng(512)
    ns = brng.choice(np.arange(64, 513, 32), size=n_inst)
    grav = brng.uniform(5.0, 10.0, n_inst)
    cor = brng.uniform(-4.0, -1.0, n_inst)
    amp = brng.uniform(0.05, 0.2, n_inst)
    # under torchrun every rank advances its share of the instances (no
    # exchange between instances); timings are max-reduced, work summed
    multi = _pkg_module("multi")
    rank, world, _ = rank_info()
    mine = multi.shard_by_cost([float(n) ** 2 for n in ns], world)[rank]
    meshes = {int(n): pda.create_full_mesh((int(n), int(n)), (-5.0, 5.0, -5.0, 5.0), 7) for n in sorted(set(ns[mine]))}
    t0 = time.perf_counter()
    probs = [pda.create_problem(meshes[int(ns[i])], pda.Swe2d.SlipWall, pda.InviscidFluxReconstruction.Weno5, 1,
                                {"gravity": grav[i], "coriolis": cor[i], "pulseMagnitude": amp[i]}, stream=stream)
             for i in mine]
    n_inst = len(mine)
    B = pda.create_batch(probs, stream=stream)
    U = B.initialCondition()
    setup_s = time.perf_counter() - t0
    tune = B.autotune(U, reps=2)
    shapes = [B.tile_shape(a) for a in range(2)]
    dt = 0.005
    B.advance_ssprk3(U, 0.0, dt, 1)  # capture + warm-up
    l0 = B.launch_count()
    if world > 1:
        torch.distributed.barrier()
    ms = _time_gpu(torch, stream, lambda: B.advance_ssprk3(U, 0.0, dt, steps), 1, warm=0)
    ms = multi.max_over_ranks(ms, device="cuda")
    launches = (B.launch_count() - l0) // steps
    cells = int(multi.sum_over_ranks(B.totalCells, device="cuda"))
    w = {"config": "batched_swe_slipwall_weno5_ssprk3_dt0.005_512_instances_n64-512",
         "instances": len(ns), "instances_per_rank": n_inst, "ranks": world,
         "total_cells": cells, "steps_timed": steps, "ms_per_step": ms / steps,
         "value": 3 * cells * steps / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s",
         "projected_500_steps_s": 500 * ms / steps * 1e-3, "launches_per_step": launches,
         "tile_shapes": {"x": shapes[0], "y": shapes[1]},
         "autotune_ms": {"x": tune[0].tolist(), "y": tune[1].tolist()}, "setup_s": setup_s}
    # the same step, one problem (one CUDA graph) at a time
    views = [B.instance(U, i) for i in range(n_inst)]
    for i, p in enumerate(probs):
        p.advance_ssprk3(views[i], 0.0, dt, 1)
    ms1 = _time_gpu(torch, stream, lambda: [p.advance_ssprk3(views[i], 0.0, dt, 1) for i, p in enumerate(probs)],
                    1, warm=0)
    w["per_instance_launch_ms_per_step"] = ms1
    w["batching_speedup"] = ms1 / (ms / steps)
    if orc is not None and rank == 0:
        nm = ns[mine]
        sample = [mine[int(i)] for i in np.argsort(nm)[[0, len(nm) // 2, len(nm) - 1]]]
        tot_cells, tot_s = 0, 0.0
        import tempfile
        for i in sample:
            n = int(ns[i])
            d = tempfile.mkdtemp()
            meshes[n].write(d)
            om = orc.mesh_load(d)
            op = orc.problem(om, 3, 0, 2, 1, {"gravity": grav[i], "coriolis": cor[i], "pulseMagnitude": amp[i]})
            Uo = op.initial_condition()
            t0 = time.perf_counter()
            op.ssprk3(Uo, 0.0, dt, 1)
            tot_s += time.perf_counter() - t0
            tot_cells += 3 * n * n
        w["cpu_baseline"] = {"value": tot_cells / tot_s / 1e9, "unit": "Gcell-updates/s", "cores": threads,
                             "kind": "port", "sample": "one SSP-RK3 step of the smallest, median and largest "
                             f"instance (n = {[int(ns[i]) for i in sample]}), {tot_s*1e3:.0f} ms"}
    del U, B, probs, views
    torch.cuda.empty_cache()
    return w


def workload_config():
    return {"workload": f"euler2d_riemann_ic2_weno5_velocity_{N_CELLS_SIDE}x{N_CELLS_SIDE}", "cells": N_CELLS_SIDE ** 2,
            "dofs": NDPC * N_CELLS_SIDE ** 2, "scheme": "WENO5+Rusanov", "boundary": "Neumann (transmissive)",
            "l2": "256 MiB write between timed steps (outside the per-step events)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer measurement (profiling runs)")
    ap.add_argument("--n", type=int, default=1024, help="cells per side (1024 = the benchmark workload)")
    ap.add_argument("--no-extra", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--workload", action="append", choices=sorted(WORKLOADS),
                    help="run only this secondary workload (repeatable; for profiling), no headline line")
    args = ap.parse_args()
    global N_CELLS_SIDE
    N_CELLS_SIDE = args.n
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import importlib
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ge = importlib.import_module("__graft_entry__")
    pda = ge.package()
    stream = torch.cuda.Stream()
    if args.workload:
        res = extra_workloads(pda, torch, stream, cpu=not args.no_cpu_baseline and rank == 0, names=args.workload)
        if rank == 0:
            print(json.dumps({"workloads": res}))
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0
    mesh, prob, Uh = build_workload(pda, torch, stream)
    cells = N_CELLS_SIDE ** 2
    with torch.cuda.stream(stream):
        U = torch.from_numpy(Uh).cuda()
        V = prob.createVelocity()
        flush = torch.empty(L2_FLUSH_BYTES // 8, dtype=torch.float64, device="cuda")
    stream.synchronize()

    def step():
        prob.velocity(U, 0.0, V)

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    # ---- timed region: K steps, per-step events, L2 flushed before each
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = prob.launch_count()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                ev[k][0].record(stream)
                step()
                ev[k][1].record(stream)
        torch.cuda.synchronize()
    launches = (prob.launch_count() - l0) // args.steps
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
        torch.distributed.barrier()
    value = world * cells / (ms * 1e-3) / 1e9

    # ---- e2e: host buffers through the C ABI (pinned), H2D + kernels + D2H
    if args.no_e2e:
        args.steps_e2e = 0
    Uhp = torch.from_numpy(Uh).pin_memory()
    Vhp = torch.empty(prob.totalDofSampleMesh(), dtype=torch.float64).pin_memory()
    import ctypes as C
    L = pda.lib()
    for _ in range(3):
        pda._check(L.pda_velocity_host(prob._h, C.c_void_p(Uhp.data_ptr()), 0.0, C.c_void_p(Vhp.data_ptr())))
    te = []
    for _ in range(args.steps if not args.no_e2e else 1):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pda._check(L.pda_velocity_host(prob._h, C.c_void_p(Uhp.data_ptr()), 0.0, C.c_void_p(Vhp.data_ptr())))
        te.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * sum(te) / len(te)
    assert torch.equal(Vhp, V.cpu()), "host-buffer path differs from the device path"

    # ---- per-kernel device times (dominant kernel) and roofline
    prof = prob.profile_velocity(U, V, reps=max(5, args.steps // 2))
    face_ms = (prof["faces_x"] + prof["faces_y"]) / 2
    hbm_peak, peak_src = measured_peaks()
    # faces kernel, one launch = one axis over N faces: reads U (32 B/cell) and
    # writes the face fluxes (32 B/face); half the cell's flops
    face_bytes = cells * (8 * NDPC) + (cells + N_CELLS_SIDE) * (8 * NDPC)
    achieved_gbs = face_bytes / (face_ms * 1e-3) / 1e9
    fp64_peak = pda.measure_fp64_peak()  # FLOP/s with an FMA counted as 2
    fp64_inst_peak = fp64_peak / 2.0      # FP64 instructions per second (DFMA/DMUL/DADD)
    ops_face_launch = cells * (FLOPS_PER_CELL - 24) / 2
    fp64_inst_face_launch = FP64_INST_PER_FACE * (N_CELLS_SIDE + 1) * N_CELLS_SIDE
    ops_ach = ops_face_launch / (face_ms * 1e-3)
    step_ops = cells * FLOPS_PER_CELL / (ms * 1e-3)

    line = {
        "metric": "FV residual Gcell/s", "value": value, "unit": "Gcell/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (Riemann IC2 + seeded U[-1e-3,1e-3] noise)", "config": workload_config(),
        "e2e": {"value": world * cells / (e2e_ms * 1e-3) / 1e9, "unit": "Gcell/s",
                "h2d_bytes_per_step": int(Uhp.numel() * 8), "d2h_bytes_per_step": int(Vhp.numel() * 8),
                "ms_per_step": e2e_ms},
        "gpu_launches": int(launches * args.steps),
        "roofline": {"bound": "hbm", "kernel": "k_faces_tile<Euler2d,Weno5,axis>",
                     "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak, "traffic": FACE_TRAFFIC_BYTES_PER_CELL * cells,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_faces_tile "
                                       "launch at 2048^2 (profiles/), scaled per cell to this launch",
                     "peak_source": peak_src,
                     "binding_roof": "fp64",
                     "fp64": {"achieved_gops": ops_ach / 1e9, "peak_ginst_per_s": fp64_inst_peak / 1e9,
                              "frac": ops_ach / fp64_inst_peak, "peak_tflops_fma2": fp64_peak / 1e12,
                              "peak_source": "measured DFMA probe (pda_measure_fp64_peak)",
                              "note": "algorithmic FP64 ops (add/mul/div/sqrt = 1) per second of the face kernel "
                                      "against the FP64 instruction issue rate; divisions, square roots and "
                                      "products by constants run on the integer pipe, so frac exceeds 1; "
                                      "pipe_frac is the FP64 pipe's own occupancy",
                              "inst_per_face": FP64_INST_PER_FACE,
                              "pipe_achieved_ginst_per_s": fp64_inst_face_launch / (face_ms * 1e-3) / 1e9,
                              "pipe_frac": fp64_inst_face_launch / (face_ms * 1e-3) / fp64_inst_peak,
                              "pipe_source": "ncu dadd + dmul + dfma thread-instruction counters of k_faces_tile "
                                             "(profiles/k_faces_tile_riemann2d_weno5_2048.md) x faces per launch "
                                             "/ live CUDA-event time",
                              "step_achieved_gops": step_ops / 1e9,
                              "algorithmic_ops_per_cell": FLOPS_PER_CELL},
                     "kernel_ms": prof},
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"], line["parity"] = cpu_baseline(Uh, V.cpu().numpy(), budget_s=args.cpu_budget)
    if not args.no_extra:
        del U, V, flush
        torch.cuda.empty_cache()
        # workloads that shard over the ranks run on every rank, first; the
        # others on rank 0 alone (the other ranks are done)
        res = extra_workloads(pda, torch, stream, cpu=not args.no_cpu_baseline and rank == 0,
                              names=[n for n in WORKLOADS if n in SHARDED])
        if rank == 0:
            res.update(extra_workloads(pda, torch, stream, cpu=not args.no_cpu_baseline,
                                       names=[n for n in WORKLOADS if n not in SHARDED]))
            line["workloads"] = res
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
