"""Benchmark: batched SG4 H.psi (FP64) on the 6-D L=8 workload, one GB300.

A step is one H.psi over the block of 20 right-hand sides of the 6-D, L=8,
Q-dependent-G (type 10) SG4 Hamiltonian (seeded synthetic data, see
elvibrot_gb300/configs.py).  value = right-hand-side H.psi applications per
second with psi resident in HBM; e2e = the same through the host-pointer C
ABI (pinned host psi copied in and H.psi copied out every step).  L2 is
flushed (256 MB write) before every timed step.  The launch plan is the
autotuner's, chosen before the warm-up (--no-tune: the automatic plan;
--plan G,R,S: a given one); the automatic plan is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm's CPU implementation of the
path (the C/OpenMP restatement in oracle/, the reference itself being
Fortran that cannot be compiled here) on all host cores, same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SG4 H·psi/s FP64 (≤1e-12 rel) batched vs plain on 1 GB300"
UNIT = "Hpsi/s"
CONFIG_INDEX = 1
WORKLOAD = "6-D SG4 (HO modes, L=LB=8, nb=l+1, nq=l+2), type-10 KEO with Q-dependent G, 20 real RHS"


def workload_config(model, nrhs, N, nb_SG, sum_nq):
    """The workload's description, identical in both arms (no device or run keys)."""
    return {"workload": WORKLOAD, "D": model.D, "L": model.L, "nrhs": nrhs, "N": int(N), "nb_SG": int(nb_SG),
            "sum_nq": int(sum_nq), "type_op": int(model.type_op)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(t, device):
    """The largest of the ranks' values (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist
    x = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def build_oracle_inputs(model):
    from oracle.oracle import OracleSG4
    O = OracleSG4(model.D, model.L, model.L, 1, 1, 2, 1, scaleQ=model.scaleQ)
    Q = O.grid_points()
    kw = dict(V=model.V(Q))
    if model.type_op == 1:
        kw.update(type_op=1, F2=model.F2.ravel())
    else:
        nq = np.prod(O.tables()[0] + 2, axis=1)
        kw.update(type_op=10, G=model.G_grid(Q, nq))
    return O, kw


def time_oracle(model, nrhs, min_seconds, min_steps, max_steps, seed, threads=None):
    """Times the CPU restatement on `threads` host threads (all by default);
    returns (Hpsi/s, steps, seconds, threads)."""
    from elvibrot_gb300.configs import random_psi
    O, kw = build_oracle_inputs(model)
    psi = random_psi(O.N, nrhs, seed)
    threads = threads or os.cpu_count() or 1
    O.hpsi(psi[:, :1], nthreads=threads, **kw)  # warm
    t0 = time.perf_counter()
    steps = 0
    while steps < min_steps or (time.perf_counter() - t0 < min_seconds and steps < max_steps):
        O.hpsi(psi, nthreads=threads, **kw)
        steps += 1
    dt = time.perf_counter() - t0
    return steps * nrhs / dt, steps, dt, threads


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=max(mx), reasons=sorted(reasons), samples=len(sm))
        return out


def profile_traffic():
    """Per-launch DRAM traffic of the H.psi kernel from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "hpsi_items_6d_l8_20rhs.txt")
    if not os.path.exists(p):
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(p).read())
    return float(m.group(1)) if m else None


def bench_davidson(op):
    """Lowest 20 levels of the benchmark operator (restart 60, residual 1e-8):
    every iteration as two recorded CUDA graphs (the default) and as the same
    steps launched one by one."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d = op.diagonal()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    # one untimed solve first: its cuBLAS calls load the library's kernels
    # (seconds on a cold page cache), which is not the solver's cost
    op.davidson(20, max_subspace=60, conv_resi=1e-8, symmetrize=True, diag=d, max_it=1000)
    res = {"levels": 20, "max_subspace": 60, "conv_resi": 1e-8, "diagonal_s": t1 - t0}
    runs = {}
    for graph in (False, True):
        torch.cuda.synchronize()
        ta = time.perf_counter()
        runs[graph] = op.davidson(20, max_subspace=60, conv_resi=1e-8, symmetrize=True, diag=d, max_it=1000,
                                  graph=graph)
        torch.cuda.synchronize()
        res["davidson_s" if graph else "davidson_eager_s"] = time.perf_counter() - ta
    ev, vec, rs, its = runs[True]
    res.update({"iterations": its, "eager_over_graph": res["davidson_eager_s"] / res["davidson_s"],
                "bit_identical_to_eager": bool(np.array_equal(ev, runs[False][0])),
                "max_residual": float(np.max(rs)), "E0_hartree": float(ev[0])})
    return res


def bench_oc_gradient():
    """Config 3: 4-D L=7, H(t) = H0 - E(t) mu, 2000 RK4 steps of 5 a.u., checkpoints
    every 45 steps; seconds per gradient evaluation and its ratio to one forward
    propagation."""
    import torch
    from elvibrot_gb300 import ParamOp
    from elvibrot_gb300.configs import config, make_dipole
    cfg = config(3)
    m = cfg["model"]
    H0 = m.operator()
    mu = ParamOp(H0.basis, 0, V_poly=make_dipole(m, cfg["seed"]))
    ev, vec, rs, its = H0.davidson(3, conv_resi=1e-10, max_it=500)
    psi0 = vec[0].to(torch.complex128).contiguous()
    target = vec[2].to(torch.complex128).contiguous()
    E = np.random.Generator(np.random.PCG64(cfg["seed"])).normal(0.0, 1e-3, size=2000)
    v = torch.randn((1, H0.basis.N), dtype=torch.float64, device="cuda")
    hv = torch.empty_like(v)
    for _ in range(60):                                  # power iteration for the top of the spectrum
        v /= torch.linalg.vector_norm(v)
        H0.hpsi_dev(v, hv)
        Hmax = float((v * hv).sum().item())
        v, hv = hv, v
    E0 = 0.5 * (float(ev[0]) + Hmax)                     # RK4 on H0 - E0 (fcn_field's para_H%E0)
    nsub = 10                                            # RK4 steps of 0.5 a.u. per 5-a.u. field sample
    res = {"workload": "4-D SG4 L=7 type 1, 2000 field samples of 5 a.u. (10 RK4 steps each), checkpoint every 45",
           "E0": E0, "Hmax_estimate": Hmax}
    out = {}
    for graph in (True, False):
        P = psi0.clone()
        H0.rk4_field(mu, E[:10], P, 5.0, E0=E0, nsub=nsub, graph=graph)  # warm
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        P = psi0.clone()
        H0.rk4_field(mu, E, P, 5.0, E0=E0, nsub=nsub, graph=graph)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        J, g = H0.oc_gradient(mu, E, psi0, target, 5.0, checkpoint=45, E0=E0, nsub=nsub, graph=graph)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        out[graph] = (P.cpu(), J, g)
        sfx = "" if graph else "_eager"
        res.update({"s_per_iter" + sfx: t2 - t1, "forward_s" + sfx: t1 - t0})
        if graph:
            res.update({"ratio_to_forward": (t2 - t1) / (t1 - t0), "J": J,
                        "norm_after_forward": float(torch.linalg.vector_norm(P).item()),
                        "us_per_rk4_stage": 1e6 * (t1 - t0) / (len(E) * nsub * 4)})
    res["graph_bit_identical_to_eager"] = bool(torch.equal(out[True][0], out[False][0]) and out[True][1] == out[False][1]
                                               and np.array_equal(out[True][2], out[False][2]))
    res["forward_eager_over_graph"] = res["forward_s_eager"] / res["forward_s"]
    res["gradient_eager_over_graph"] = res["s_per_iter_eager"] / res["s_per_iter"]
    return res


def coherent_packets(D, L, scaleQ, nrhs, shift=1.0):
    """(nrhs, N) complex packets: coherent states of mode 1 displaced by `shift`
    along Q1 (momentum 0.25 j in the dimensionless units of packet j), the other
    modes in their ground state, in the packed basis (sum n_i <= L, last index
    fastest, so (n, 0, ..., 0) sits after every tuple whose first index is < n)."""
    from math import comb, factorial
    N = comb(L + D, D)
    pos = [0]
    for m in range(L):
        pos.append(pos[-1] + comb(L - m + D - 1, D - 1))
    out = np.zeros((nrhs, N), dtype=np.complex128)
    for j in range(nrhs):
        a = scaleQ[0] * shift * (1.0 + 0.25j * j) / np.sqrt(2.0)
        c = np.array([a ** n / np.sqrt(float(factorial(n))) for n in range(L + 1)])
        out[j, pos] = c / np.linalg.norm(c)
    return out


def bench_uneven(seconds_cap=90.0):
    """Uneven-instance batching: 64 seeded Hamiltonians (D in 3..9, L in 4..10,
    type 1), 8 complex packets each.  Times one merged H.psi over all of them
    (evr_sg4_multi_hpsi) against one evr_sg4_hpsi_cplx launch per instance,
    and one order-30 Chebyshev step of dt = 10 a.u. in lock-step."""
    import torch
    from elvibrot_gb300 import MultiOp
    from elvibrot_gb300.configs import uneven_instances
    t0 = time.perf_counter()
    models = uneven_instances(64)
    ops = [m.operator() for m in models]
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    n = len(ops)
    nrhs = 8
    flops = sum(op.flops_per_rhs for op in ops) * 2 * nrhs
    # spectral bounds by power iteration on H and on Hmax - H (one real vector per instance)
    p1 = MultiOp(ops, [1] * n)
    g = torch.Generator(device="cpu").manual_seed(5)
    v = [torch.randn((1, op.basis.N), generator=g, dtype=torch.float64).cuda() for op in ops]
    hv = [torch.empty_like(x) for x in v]
    top = np.zeros(n)
    for _ in range(40):
        v = [x / torch.linalg.vector_norm(x) for x in v]
        p1.hpsi(v, hv)
        top = np.array([float((a * b).sum()) for a, b in zip(v, hv)])
        v, hv = hv, v
    Hmax = top * 1.1
    v = [torch.randn((1, op.basis.N), generator=g, dtype=torch.float64).cuda() for op in ops]
    low = np.zeros(n)
    for _ in range(40):                                  # (H - E0) psi / Esc with Esc = -1: (Hmax - H) psi
        v = [x / torch.linalg.vector_norm(x) for x in v]
        p1.hpsi(v, hv, E0=list(Hmax), Esc=[-1.0] * n)
        low = Hmax - np.array([float((a * b).sum()) for a, b in zip(v, hv)])
        v, hv = hv, v
    Hmin = low - 0.1 * (Hmax - low)
    psis = [torch.from_numpy(coherent_packets(m.D, m.L, m.scaleQ, nrhs)).cuda() for m in models]
    outs = [torch.empty_like(P) for P in psis]
    plan = MultiOp(ops, [nrhs] * n, complex_=True)
    plan.hpsi(psis, outs)                                # warm
    torch.cuda.synchronize()
    reps = 3
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        plan.hpsi(psis, outs)
    b.record()
    torch.cuda.synchronize()
    multi_s = a.elapsed_time(b) / 1e3 / reps
    ref = [torch.empty_like(P) for P in psis]
    for op, P, O in zip(ops, psis, ref):                  # warm the per-instance work lists
        op.hpsi_dev(P, O)
    torch.cuda.synchronize()
    a.record()
    for op, P, O in zip(ops, psis, ref):
        op.hpsi_dev(P, O)
    b.record()
    torch.cuda.synchronize()
    seq_s = a.elapsed_time(b) / 1e3
    same = all(torch.equal(x, y) for x, y in zip(outs, ref))
    res = {"workload": "64 uneven type-1 instances (D 3..9, L 4..10, sum N %d), 8 complex packets each"
                       % sum(op.basis.N for op in ops),
           "setup_s": setup_s, "flops_per_multi_hpsi": flops,
           "multi_hpsi_s": multi_s, "per_instance_launches_s": seq_s, "multi_over_per_instance": seq_s / multi_s,
           "multi_tflops": flops / multi_s / 1e12, "bitwise_equal_to_per_instance": bool(same)}
    if 29 * multi_s < seconds_cap:
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ac = plan.cheby_propagate(psis, list(Hmin), list(Hmax), 10.0, 30, 1)
        torch.cuda.synchronize()
        step_s = time.perf_counter() - t1
        norms = [float(torch.linalg.vector_norm(P, dim=1).sub(1.0).abs().max()) for P in psis]
        res.update({"cheby_order": 30, "cheby_dt": 10.0, "cheby_step_s": step_s,
                    "cheby_200_steps_s_estimate": 200 * step_s, "max_norm_drift": max(norms),
                    "autocorr_t10_first": [float(ac[0][1, 0].real), float(ac[0][1, 0].imag)]})
    return res


def bench_config0(reps=200):
    """The 3-D L=6 type-1 workload (one real vector): batched and per-term GPU
    H.psi, the CPU restatement on all host threads, the largest relative
    difference from it, and Davidson for the lowest 10 levels."""
    import torch
    from elvibrot_gb300.configs import config, random_psi
    cfg = config(0)
    m = cfg["model"]
    op = m.operator()
    N = op.basis.N
    psi = random_psi(N, 1, cfg["seed"])
    P = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    H = torch.empty_like(P)
    res = {"workload": "3-D SG4 L=6 type 1 (constant G), 1 real vector", "N": N, "nb_SG": op.basis.nb_SG}
    for plain in (False, True):
        op.hpsi_dev(P, H, plain=plain)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            op.hpsi_dev(P, H, plain=plain)
        b.record()
        torch.cuda.synchronize()
        res["plain_hpsi_per_s" if plain else "batched_hpsi_per_s"] = reps / (a.elapsed_time(b) / 1e3)
    op.hpsi_dev(P, H)
    got = H.cpu().numpy().T
    O, kw = build_oracle_inputs(m)
    ref = O.hpsi(psi, **kw)
    res["max_rel_err_vs_cpu"] = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    v, steps, dt, threads = time_oracle(m, 1, min_seconds=0.5, min_steps=3, max_steps=2000, seed=cfg["seed"])
    res.update({"cpu_hpsi_per_s": v, "cpu_threads": threads})
    ev, vec, rs, its = op.davidson(10, conv_resi=1e-9, max_it=300)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev, vec, rs, its = op.davidson(10, conv_resi=1e-9, max_it=300)
    torch.cuda.synchronize()
    res.update({"davidson_10_levels_s": time.perf_counter() - t0, "davidson_iterations": its,
                "lowest_levels_hartree": [float(x) for x in ev[:3]]})
    return res


def bench_cheby_graph(nsteps=200):
    """Fixed-order Chebyshev (order 30, dt = 10 a.u.) of one complex packet on the
    4-D L=7 type-1 system: every step eagerly launched vs replayed from a CUDA
    graph recorded once (the launch-bound regime of small operators)."""
    import torch
    from elvibrot_gb300.configs import config
    m = config(3)["model"]
    op = m.operator()
    N = op.basis.N
    v = torch.randn((1, N), dtype=torch.float64, device="cuda")
    hv = torch.empty_like(v)
    top = 1.0
    for _ in range(60):
        v /= torch.linalg.vector_norm(v)
        op.hpsi_dev(v, hv)
        top = float((v * hv).sum().item())
        v, hv = hv, v
    Hmin, Hmax = 0.0, 1.1 * top
    g = torch.Generator(device="cpu").manual_seed(3)
    P0 = torch.randn((1, N), generator=g, dtype=torch.complex128).cuda()
    P0 /= torch.linalg.vector_norm(P0)
    res = {"workload": f"4-D SG4 L=7 type 1, 1 complex packet, order 30, dt 10 a.u., {nsteps} steps"}
    out = {}
    for graph in (False, True):
        P = P0.clone()
        op.cheby_propagate(P, Hmin, Hmax, 10.0, npoly=30, nsteps=3, graph=graph)   # warm
        P = P0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op.cheby_propagate(P, Hmin, Hmax, 10.0, npoly=30, nsteps=nsteps, graph=graph)
        torch.cuda.synchronize()
        res["graph_s" if graph else "eager_s"] = time.perf_counter() - t0
        out[graph] = P
    res["eager_over_graph"] = res["eager_s"] / res["graph_s"]
    res["bit_identical"] = bool(torch.equal(out[False], out[True]))
    return res


def _terms_array(D, L):
    """Smolyak terms l (|l| in [max(0, L-D+1), L]) as an int array, and their grid sizes prod(l+2)."""
    Lmin = max(0, L - D + 1)
    rows = []

    def rec(prefix, rem):
        if len(prefix) == D - 1:
            for v in range(rem + 1):
                if L - rem + v >= Lmin:
                    rows.append(prefix + (v,))
            return
        for v in range(rem + 1):
            rec(prefix + (v,), rem - v)
    rec((), L)
    l = np.array(rows, dtype=np.int64)
    return l, np.prod(l + 2, axis=1).astype(np.float64)


def type10_flops_per_rhs(D, L):
    """evr_sg4_flops_per_rhs for a type-10 operator with V and G (nb = l+1, nq = l+2), without
    building the basis: the basis<->grid passes in the kernel's mode order (larger l first, ties by
    index), the derivative passes (4 q sum nq_i), the G contraction (2 D^2 q), V.x (q), the single
    multiply-add closing pass B (2 q) and the weighted scatter (2 nb)."""
    l, q = _terms_array(D, L)
    nb, nq = (l + 1).astype(np.float64), (l + 2).astype(np.float64)
    order = np.argsort(-l, axis=1, kind="stable")
    f = np.zeros(len(l))
    rows = np.arange(len(l))
    for direction in (0, 1):
        cur = (nb if direction == 0 else nq).copy()
        seq = range(D) if direction == 0 else range(D - 1, -1, -1)
        for k in seq:
            i = order[:, k]
            rest = np.prod(cur, axis=1) / cur[rows, i]
            f += 2.0 * nb[rows, i] * nq[rows, i] * rest
            cur[rows, i] = (nq if direction == 0 else nb)[rows, i]
    f += 4.0 * q * nq.sum(axis=1) + 2.0 * D * D * q + q + 2.0 * q + 2.0 * np.prod(nb, axis=1)
    return float(f.sum())


def bench_streamed_12d(L=6, nrhs=32, budget_gib=64):
    """The 12-D workload shape (type 10 with Q-dependent G, 32 complex packets)
    at Smolyak level L: its V and G (sum_nq x 145 doubles) exceed the device,
    so they are evaluated per slice of Smolyak terms inside every H.psi.
    Times one H.psi and extrapolates to L=10 by the flop count."""
    import torch
    from elvibrot_gb300.configs import SEED0, make_model
    m = make_model(12, L, 10, SEED0 + 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    op = m.operator(field_budget=budget_gib << 30)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    N, snq = op.basis.N, op.basis.sum_nq
    g = torch.Generator(device="cpu").manual_seed(4)
    P = (torch.randn((nrhs, N), generator=g, dtype=torch.float64)
         + 1j * torch.randn((nrhs, N), generator=g, dtype=torch.float64)).cuda()
    P /= torch.linalg.vector_norm(P, dim=1, keepdim=True)
    O = torch.empty_like(P)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    op.hpsi_dev(P, O)
    b.record()
    torch.cuda.synchronize()
    t = a.elapsed_time(b) / 1e3
    flops = op.flops_per_rhs * 2 * nrhs
    D = 12
    vmul = sum(int(np.sum(e)) for e in m.V.expo)
    field_flops = snq * (2.0 * D ** 3 + vmul + len(m.V.coef))               # affine G, V polynomial
    fL, f10 = type10_flops_per_rhs(D, L), type10_flops_per_rhs(D, 10)
    return {"workload": f"12-D SG4 L={L} type 10, Q-dependent G, {nrhs} complex packets, fields streamed",
            "N": N, "sum_nq": snq, "field_bytes_resident": snq * 8 * (1 + D * D), "field_budget": budget_gib << 30,
            "slices": op.field_slices, "setup_s": setup_s, "hpsi_s": t, "hpsi_flops": flops,
            "flops_per_rhs_check": [op.flops_per_rhs, fL],
            "field_eval_flops": field_flops, "tflops_hpsi_only": flops / t / 1e12,
            "tflops_with_fields": (flops + field_flops) / t / 1e12,
            "L10_hpsi_s_estimate": t * f10 / fL, "L10_sum_nq": float(_terms_array(D, 10)[1].sum())}


def bench_streamed_12d_l10(nrhs=1, budget_gib=64):
    """The 12-D workload at its stated level, L=10 (646,646 Smolyak terms,
    6.8e10 grid points; V and G would take 79 TB), on nrhs real vectors: one
    H.psi with the fields evaluated slice by slice inside it.  Minutes of GPU
    time, so only on request (--extras stream12_L10)."""
    import torch
    from elvibrot_gb300.configs import SEED0, make_model
    m = make_model(12, 10, 10, SEED0 + 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    op = m.operator(field_budget=budget_gib << 30)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    N, snq = op.basis.N, op.basis.sum_nq
    g = torch.Generator(device="cpu").manual_seed(10)
    P = torch.randn((nrhs, N), generator=g, dtype=torch.float64).cuda()
    P /= torch.linalg.vector_norm(P, dim=1, keepdim=True)
    O = torch.empty_like(P)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    op.hpsi_dev(P, O)
    b.record()
    torch.cuda.synchronize()
    t = a.elapsed_time(b) / 1e3
    D = 12
    flops = op.flops_per_rhs * nrhs
    vmul = sum(int(np.sum(e)) for e in m.V.expo)
    field_flops = snq * (2.0 * D ** 3 + vmul + len(m.V.coef))
    return {"workload": f"12-D SG4 L=10 type 10, Q-dependent G, {nrhs} real vector(s), fields streamed",
            "N": N, "nb_SG": op.basis.nb_SG, "sum_nq": snq, "field_bytes_resident": snq * 8 * (1 + D * D),
            "field_budget": budget_gib << 30, "slices": op.field_slices, "setup_s": setup_s, "hpsi_s": t,
            "hpsi_flops": flops, "field_eval_flops": field_flops, "tflops_with_fields": (flops + field_flops) / t / 1e12,
            "flops_per_rhs_library": op.flops_per_rhs, "flops_per_rhs_formula": type10_flops_per_rhs(D, 10),
            "finite": bool(torch.isfinite(O).all().item())}


def bench_davidson12(L=4, nev=50):
    """The 12-D workload's Davidson (50 levels) at a level where the dense
    operator can still check it: type 10 with Q-dependent G, L=4 (N = 1820),
    symmetrised, residual 1e-8, the term-wise diagonal as preconditioner; the
    levels against a dense diagonalisation of (H + H^T)/2 built from the GPU
    operator.  About a minute, so only on request (--extras davidson12)."""
    import torch
    from elvibrot_gb300.configs import SEED0, make_model
    CM1 = 4.556335252767e-6
    m = make_model(12, L, 10, SEED0 + 4)
    op = m.operator()
    N = op.basis.N
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d = op.diagonal()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ev, vec, rs, its = op.davidson(nev, block=nev, max_subspace=3 * nev, conv_resi=1e-8, symmetrize=True, diag=d,
                                   max_it=2000)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    H = np.empty((N, N))
    for n0 in range(0, N, 256):
        k = min(256, N - n0)
        E = torch.zeros((k, N), dtype=torch.float64, device="cuda")
        E[torch.arange(k), torch.arange(n0, n0 + k)] = 1.0
        out = torch.empty_like(E)
        op.hpsi_dev(E, out)
        H[:, n0:n0 + k] = out.cpu().numpy().T
    ref = np.linalg.eigvalsh(0.5 * (H + H.T))[:nev]
    return {"workload": f"12-D SG4 L={L} type 10 (Q-dependent G), lowest {nev} levels of (H + H^T)/2",
            "N": N, "diagonal_s": t1 - t0, "davidson_s": t2 - t1, "iterations": its, "max_residual": float(np.max(rs)),
            "max_dev_from_dense_cm1": float(np.max(np.abs(ev - ref)) / CM1)}


def run_ours(args, ws, rank, local):
    import torch
    import torch.distributed as dist
    from elvibrot_gb300 import fp64_peak_tflops, lib
    from elvibrot_gb300.configs import config, random_psi

    torch.cuda.set_device(local)
    cfg = config(CONFIG_INDEX)
    model, nrhs = cfg["model"], cfg["nrhs"]
    op = model.operator()
    N = op.basis.N
    psi_np = random_psi(N, nrhs, cfg["seed"])
    psi = torch.from_numpy(np.ascontiguousarray(psi_np.T)).cuda()
    out = torch.empty_like(psi)
    flush = torch.empty(32 * 1024 * 1024, dtype=torch.float64, device="cuda")  # 256 MB > L2
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    def step():
        op.hpsi_dev(psi, out, stream=sh)

    # the autotuner picks the launch plan before anything is timed, as the
    # reference runs Tune_SG4threads_HPsi before its propagations and
    # diagonalisations (SRC/sub_main/vib.f90:370,583); --no-tune keeps the
    # automatic plan
    tr = None
    if args.plan:
        op.set_plan(*[int(x) for x in args.plan.split(",")])
    elif not args.no_tune:
        tr = op.tune_plan(nrhs)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    peak = fp64_peak_tflops()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    launches = op.last_launches * args.steps
    ms = [a.elapsed_time(b) for a, b in ev]
    t_tot = sum(ms) / 1e3
    if ws > 1:
        t_tot = max_over_ranks(t_tot, "cuda")
        dist.barrier()
    ms_step = 1e3 * t_tot / args.steps
    value = ws * args.steps * nrhs / t_tot

    # end to end through the host-pointer C ABI: pinned psi in, H.psi out, every step
    ph = torch.from_numpy(np.ascontiguousarray(psi_np.T)).pin_memory()
    hh = torch.empty_like(ph).pin_memory()
    L = lib()
    import ctypes
    for _ in range(2):
        L.evr_sg4_hpsi_host(op._h, nrhs, ctypes.c_void_p(ph.data_ptr()), N, ctypes.c_void_p(hh.data_ptr()), N, 0.0, 1.0)
    e2e_t = 0.0
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = L.evr_sg4_hpsi_host(op._h, nrhs, ctypes.c_void_p(ph.data_ptr()), N, ctypes.c_void_p(hh.data_ptr()), N,
                                 0.0, 1.0)
        e2e_t += time.perf_counter() - t0
        assert rc == 0, L.evr_sg4_last_error().decode()
    np.testing.assert_allclose(hh.numpy(), out.cpu().numpy(), rtol=0, atol=1e-12 * float(out.abs().max()))
    e2e_value = ws * args.steps * nrhs / e2e_t

    # the automatic plan on the same workload and protocol, for comparison
    auto = None
    if tr is not None or args.plan:
        op.set_plan()
        step()  # untimed: the first call under a new plan builds its work list
        torch.cuda.synchronize()
        ta = 0.0
        for k in range(args.steps):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize()
            ta += a.elapsed_time(b) / 1e3
        auto = {"value": ws * args.steps * nrhs / ta, "unit": UNIT, "ms_per_step": 1e3 * ta / args.steps}

    # plain per-term path (one launch per Smolyak term) on the same workload
    plain_steps = max(2, min(5, args.steps))
    op.hpsi_dev(psi, out, plain=True)
    torch.cuda.synchronize()
    pt = 0.0
    for k in range(plain_steps):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        op.hpsi_dev(psi, out, stream=sh, plain=True)
        b.record(stream)
        torch.cuda.synchronize()
        pt += a.elapsed_time(b) / 1e3
    plain_value = plain_steps * nrhs / pt

    # callers of the path: Davidson on the same operator, OC gradient on the 4-D L=7 system
    extras = {}
    if not args.no_extras:
        want = set(args.extras.split(","))
        if "config0" in want:
            extras["config0"] = bench_config0()
        if "davidson" in want:
            extras["davidson"] = bench_davidson(op)
        if "oc" in want:
            extras["oc_gradient"] = bench_oc_gradient()
        if "uneven" in want:
            extras["uneven_instances"] = bench_uneven()
        if "graph" in want:
            extras["cheby_graph"] = bench_cheby_graph()
        if "stream12" in want:
            extras["streamed_12d"] = bench_streamed_12d()
        if "davidson12" in want:
            extras["davidson12"] = bench_davidson12()
        if "stream12_L10" in want:
            extras["streamed_12d_L10"] = bench_streamed_12d_l10()

    flops = op.flops_per_rhs * nrhs
    achieved = flops / (ms_step / 1e3) / 1e12
    b = op.basis
    D = model.D
    alg_bytes = 8.0 * 2 * N * nrhs + 8.0 * b.sum_nq * (1 + D * D)
    hbm_peak = None
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    hbm_peak = hbm_peak or 6800.0
    result = None
    if rank == 0:
        cpu_v, cpu_steps, cpu_dt, cpu_threads = time_oracle(model, nrhs, min_seconds=1.5, min_steps=1,
                                                            max_steps=50, seed=cfg["seed"])
        cpu1_v, cpu1_steps, cpu1_dt, _ = time_oracle(model, nrhs, min_seconds=0.0, min_steps=1, max_steps=1,
                                                     seed=cfg["seed"], threads=1)
        clocks = clk.summary()
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64; 6-D L=8 SG4 shapes, 20 RHS)",
            "config": workload_config(model, nrhs, N, b.nb_SG, b.sum_nq),
            "l2": "flushed (256 MB write) before every timed step",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * N * nrhs,
                    "d2h_bytes_per_step": 8 * N * nrhs},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": profile_traffic(),
                         "peak_source": "in-run DFMA probe (evr_probe_fp64_peak); MEASURED_PEAKS.json has no FP64 entry",
                         "flops_per_launch": flops,
                         "hbm": {"achieved": alg_bytes / (ms_step / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                                 "frac": alg_bytes / (ms_step / 1e3) / 1e9 / hbm_peak,
                                 "alg_bytes_per_launch": alg_bytes}},
            "plain": {"value": plain_value, "unit": UNIT, "steps": plain_steps,
                      "launches_per_step": 2 + b.nb_SG, "batched_over_plain": value / ws / plain_value},
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cpu_threads, "kind": "port",
                             "sample": f"{cpu_steps} full 20-RHS H.psi of the same workload in {cpu_dt:.2f} s "
                                       f"(C/OpenMP restatement, OpenMP static over Smolyak terms)"},
            "cpu_baseline_1thread": {"value": cpu1_v, "unit": UNIT, "cores": 1, "kind": "port",
                                     "sample": f"{cpu1_steps} full 20-RHS H.psi in {cpu1_dt:.2f} s, one thread "
                                               f"(the reference's serial per-term loop)"},
            "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"]},
            "gpu_launches": launches,
        }
        if tr is not None:
            result["plan"] = {"source": "autotuner (evr_sg4_tune_plan), before the warm-up", "geo": tr["geo"],
                              "rmax": tr["rmax"], "split": tr["split"], "tuner_best_ms": tr["ms"],
                              "tuner_automatic_ms": tr["default_ms"]}
            result["automatic_plan"] = auto
        elif args.plan:
            g, r, sp = [int(x) for x in args.plan.split(",")]
            result["plan"] = {"source": "given (--plan)", "geo": g, "rmax": r, "split": sp}
            result["automatic_plan"] = auto
        else:
            result["plan"] = {"source": "automatic (--no-tune)"}
        result.update(extras)
    return result


def run_reference(args, ws, rank):
    from elvibrot_gb300.configs import config
    if rank != 0:
        return None
    cfg = config(CONFIG_INDEX)
    model, nrhs = cfg["model"], cfg["nrhs"]
    from oracle.oracle import OracleSG4  # noqa: F401
    O, kw = build_oracle_inputs(model)
    from elvibrot_gb300.configs import random_psi
    psi = random_psi(O.N, nrhs, cfg["seed"])
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.hpsi(psi[:, :2], nthreads=threads, **kw)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.hpsi(psi, nthreads=threads, **kw)
    dt = time.perf_counter() - t0
    v = args.steps * nrhs / dt
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded PCG64; 6-D L=8 SG4 shapes, 20 RHS)", "impl": "reference",
            "config": workload_config(model, nrhs, O.N, len(O.tables()[0]),
                                      int(np.prod(O.tables()[0] + 2, axis=1).sum())),
            "parallelism": f"{threads} host threads",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full 20-RHS H.psi steps (the reference is Fortran with no "
                                       f"compiler on this image; timed: its C/OpenMP restatement)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="skip the timings of the callers")
    ap.add_argument("--no-tune", action="store_true", help="keep the automatic launch plan (no autotuner)")
    ap.add_argument("--plan", default="", help="a fixed launch plan 'geo,rmax,split' instead of the autotuner's "
                                                "(geo 0 wide, 1 narrow, 2 mid; for reproducible profiles)")
    ap.add_argument("--extras", default="config0,davidson,oc,uneven,graph,stream12",
                    help="callers to time: config0 (the 3-D L=6 workload), davidson, oc (optimal-control gradient), "
                         "uneven (64-instance batching), "
                         "graph (Chebyshev steps replayed from a CUDA graph), stream12 (12-D type 10, streamed fields); "
                         "also on request: stream12_L10 (the 12-D workload at L=10, minutes), davidson12 (50 levels of "
                         "the 12-D operator at L=4, checked against dense diagonalisation)")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        import torch
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        res = run_reference(args, ws, rank)
    else:
        res = run_ours(args, ws, rank, local)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
