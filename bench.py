#!/usr/bin/env python
"""Benchmark of the two-site DMRG sweep on one GB300.

Workload: open spin-1/2 Heisenberg chain H = sum (Sx Sx + Sy Sy + Delta Sz Sz),
L=64, Delta=1, d=2, MPO bond dimension 5; seeded Gaussian initial MPS (bond
dimensions min(2^k, 2^(L-k), 64), right-normalised); chi_max ramped
64 -> 256 -> 1024, 24 Lanczos steps per bond, no weight-based truncation
(eps_trunc = 0: every bond keeps min(d^k, d^(L-k), chi_max) states, so the
timed sweeps really run at chi = 1024).

A "step" is one full sweep (L->R then R->L, 126 local updates) at chi_max=1024.
The W warm-up steps are the ramp sweeps (chi 64, 256, then 1024); the K timed
sweeps run in one dmrg_two_site call at chi_max=1024.  Inputs (environments,
Krylov bases, MPS at chi=1024) are far larger than the 129 MB L2.

Reported (one JSON line on rank 0):
  value          seconds per sweep, device time (CUDA events), inputs resident
  e2e            the same through the C ABI from pinned host buffers
                 (MPS/MPO copied in and the final MPS + energy copied out
                 inside the timed region)
  heff_tflops    algorithmic H_eff FLOP/s over the whole Lanczos phase
  roofline       the tcgen05 TF32x3 GEMM: every launch of the timed sweeps,
                 timed with CUDA events on the launching stream; algorithmic
                 FLOP/s vs the measured-BF16-derived 3xTF32 ceiling
  breakdown      CUDA-event seconds of the timed sweeps per phase (H_eff
                 applies, other Lanczos work, subspace / Jacobi splits, envs)
  fp64           the plain FP64 form: centre-bond H_eff apply time and an
                 accuracy check |dE/E| (mixed vs FP64) on the same ramp to chi=256
  cpu_baseline   the CPU FP64 oracle (NumPy/LAPACK, all host cores) on one
                 centre-bond local update, extrapolated to a sweep by FLOPs

``--impl reference`` times the CPU oracle port of the reference path instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

# The reference arm times the CPU oracle with every host core.  A launcher that pins BLAS to
# one thread per rank (torchrun sets OMP_NUM_THREADS=1) is overridden here, before NumPy
# loads its BLAS; only rank 0 of that arm does any work.
def _impl_from_argv(argv):
    for k, a in enumerate(argv):
        if a == "--impl" and k + 1 < len(argv):
            return argv[k + 1]
        if a.startswith("--impl="):
            return a.split("=", 1)[1]
    return "ours"


if _impl_from_argv(sys.argv[1:]) == "reference":
    for _var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[_var] = str(os.cpu_count() or 1)

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

L_SITES = 64
D_PHYS = 2
MPO_D = 5
LANCZOS = 24
EPS = 0.0
RAMP = [64, 256, 1024]
# accuracy check (mixed vs FP64): sweeps at chi=256 until both forms converge, so
# the difference measures precision rather than early-trajectory noise
ACC_RAMP = (64, 256, 256, 256, 256)
# dram__bytes_read.sum + dram__bytes_write.sum of one centre-bond H_eff GEMM launch
# (5120 x 4096 x 1024 at chi=1024, 128x224 tiles) from an ncu --set full capture
TC_GEMM_TRAFFIC_BYTES = (80.092 + 47.428) * 1e6
METRIC = "DMRG sweep s & H_eff TFLOP/s, mixed-prec vs FP64 on GPU at |dE/E|<=1e-9"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--prec", default="tf32x3", choices=["tf32x3", "fp64"])
    ap.add_argument("--chi", type=int, default=1024)
    ap.add_argument("--L", type=int, default=L_SITES)
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64/roofline/CPU side measurements")
    ap.add_argument("--verbose", action="store_true", help="log every split of the timed sweeps to stderr")
    ap.add_argument("--mode", default="sweep",
                    choices=["sweep", "heff", "heff-grid", "split", "hubbard", "contractions", "fp64-ref",
                             "lanczos", "fp64tc"],
                    help="heff / split: only centre-bond H_eff applies / warm splits (small, fixed workloads "
                         "for profilers); heff-grid: H_eff over chi x D x d; contractions: the MPS/MPO "
                         "contraction operations of the reference's contraction benchmark")
    ap.add_argument("--nsites", type=int, default=6, help="contractions: number of sites")
    ap.add_argument("--d", type=int, default=2, help="contractions: physical dimension")
    ap.add_argument("--runs", type=int, default=3, help="contractions: timed repetitions per operation")
    ap.add_argument("--jsonl", default="", help="contractions: append one JSONL record per operation here")
    ap.add_argument("--ramp-sweeps", default="", help="hubbard: sweeps per ramp stage, e.g. 1,1,1,1")
    ap.add_argument("--out", default="", help="fp64-ref: also write the JSON line to this file")
    ap.add_argument("--forms", default="fp64,tf32x3", help="fp64-ref: forms to run")
    return ap.parse_args()


def heff_mode(args):
    """W + K centre-bond H_eff applies at (chi, D=5, d=2); one JSON line (profiling workload)."""
    import torch
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300 import _lib
    ctx = ct.get_context(0)
    chi = args.chi
    mpo = ct.create_spin_half_xxz_mpo(ctx, 8, 1.0)
    W = mpo.sites[3]
    g = torch.Generator(device="cpu").manual_seed(5)
    dev = ctx.torch_device
    th = ct.DenseTensor(torch.randn(chi * 4 * chi, generator=g, dtype=torch.float64).to(dev), [chi, 2, 2, chi])
    Le = ct.DenseTensor(torch.randn(MPO_D * chi * chi, generator=g, dtype=torch.float64).to(dev), [MPO_D, chi, chi])
    Re = ct.DenseTensor(torch.randn(MPO_D * chi * chi, generator=g, dtype=torch.float64).to(dev), [MPO_D, chi, chi])
    for _ in range(args.warmup):
        ct.apply_two_site_heff(th, Le, Re, W, W, ctx, prec=args.prec)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = _lib.launch_count()
    e0.record()
    for _ in range(args.steps):
        ct.apply_two_site_heff(th, Le, Re, W, W, ctx, prec=args.prec)
    e1.record()
    torch.cuda.synchronize()
    s = e0.elapsed_time(e1) * 1e-3 / max(args.steps, 1)
    F = heff_flops(chi, chi)
    print(json.dumps({"metric": "H_eff apply seconds", "value": s, "unit": "s/apply", "tflops": F / s / 1e12,
                      "dtype": args.prec, "config": {"workload": f"centre-bond H_eff chi={chi} D=5 d=2"},
                      "steps": args.steps, "warmup": args.warmup,
                      "gpu_launches": _lib.launch_count() - n0}), flush=True)


def fp64tc_mode(args):
    """FP64 GEMM on the BF16 tensor cores (CT_PREC_FP64_TC) against the FP64 SIMT GEMM.

    GEMM shapes of the mixed form's FP64 work: the subspace split's Gram matrix
    (1024 x 1024 x 2048, Z Z^T) and its triangular product (1024 x 2048 x 1024),
    and the two products of one FP64 environment step at chi=1024, D=5, d=2
    (5120 x 2048 x 1024 and 5120 x 1024 x 2048); N(0,1) operands, seed 13.
    Per shape and form: one warm-up and --steps timed launches (CUDA events),
    FP64-equivalent TFLOP/s (2 M N K), and the largest |C_tc - C_fp64| over
    sum_k |A||B|.  Then <psi|H|psi>/<psi|psi> of a random (unnormalised) MPS,
    L=24 with bonds up to chi=1024 (Heisenberg MPO), in both forms.  One JSON line.
    """
    import ctypes as C
    import torch
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300 import _lib
    ctx = ct.get_context(0)
    dev = ctx.torch_device
    g = torch.Generator(device="cpu").manual_seed(13)
    rows = []
    for (m, n, k, tb, name) in ((1024, 1024, 2048, 1, "split Gram Z Z^T"), (1024, 2048, 1024, 0, "split L^-1 Z"),
                                (5120, 2048, 1024, 0, "env step product 1"), (5120, 1024, 2048, 0, "env step product 2")):
        A = torch.randn(m, k, generator=g, dtype=torch.float64).to(dev)
        B = (torch.randn(n, k, generator=g, dtype=torch.float64) if tb else
             torch.randn(k, n, generator=g, dtype=torch.float64)).to(dev)
        row = {"shape": [m, n, k], "what": name}
        out = {}
        for prec in (0, 2):
            Cm = torch.zeros(m, n, dtype=torch.float64, device=dev)

            def call():
                ctx.call("ct_gemm", prec, 0, tb, m, n, k, C.c_double(1.0), C.c_void_p(A.data_ptr()), k,
                         C.c_void_p(B.data_ptr()), B.shape[1], C.c_double(0.0), C.c_void_p(Cm.data_ptr()), n)
            call()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(max(args.steps, 1)):
                call()
            e1.record()
            torch.cuda.synchronize()
            sec = e0.elapsed_time(e1) * 1e-3 / max(args.steps, 1)
            out[prec] = Cm.clone()
            row["fp64_tc" if prec else "fp64"] = {"ms": sec * 1e3, "tflops": 2.0 * m * n * k / sec / 1e12}
        scale = A.abs() @ (B.abs().T if tb else B.abs())
        row["max_err_over_AB"] = float(((out[2] - out[0]).abs() / scale).max())
        row["speedup"] = row["fp64"]["ms"] / row["fp64_tc"]["ms"]
        rows.append(row)
        del A, B, out, scale
        torch.cuda.empty_cache()
    # expectation value chain
    L, chi = 24, 1024
    dims = [min(chi, 2 ** min(i, L - i)) for i in range(L + 1)]
    sites = [ct.MPSSite(ct.DenseTensor(torch.randn(dims[i] * 2 * dims[i + 1], generator=g,
                                                   dtype=torch.float64).to(dev) / math.sqrt(2 * dims[i + 1]),
                                       [dims[i], 2, dims[i + 1]])) for i in range(L)]
    mps = ct.MatrixProductState(sites)
    mpo = ct.create_spin_half_xxz_mpo(ctx, L, 1.0)
    ev = {}
    for prec in ("fp64", "fp64_tc"):
        ct.expectation_value_normalized(mps, mpo, ctx, prec=prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev[prec] = (ct.expectation_value_normalized(mps, mpo, ctx, prec=prec), None)
        torch.cuda.synchronize()
        ev[prec] = (ev[prec][0], time.perf_counter() - t0)
    print(json.dumps({"metric": "FP64 GEMM on BF16 tensor cores vs FP64 SIMT", "unit": "TFLOP/s (FP64-equivalent)",
                      "data": "synthetic", "steps": args.steps,
                      "config": {"workload": "GEMM shapes of the mixed form's FP64 work, N(0,1) seed 13; "
                                             f"<H> of a random MPS L={L} chi<={chi}"},
                      "gemm": rows,
                      "expectation": {"L": L, "chi": chi,
                                      "fp64": {"value": ev["fp64"][0], "s": ev["fp64"][1]},
                                      "fp64_tc": {"value": ev["fp64_tc"][0], "s": ev["fp64_tc"][1]},
                                      "rel_diff": abs(ev["fp64_tc"][0] - ev["fp64"][0]) / abs(ev["fp64"][0])}}),
          flush=True)


def lanczos_mode(args):
    """W + K centre-bond Lanczos runs (ct_lanczos2, 24 steps, reorthogonalised) at
    (chi, D=5, d=2) on random symmetric L, R [5, chi, chi], W [5, 2, 2, 5] and theta
    (profiling workload).  Reports seconds per run, the H_eff share, and the
    Krylov vector work's algorithmic bytes over its CUDA-event time (GB/s).  One
    JSON line."""
    import ctypes as C
    import torch
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300 import _lib
    ctx = ct.get_context(0)
    chi = args.chi
    mpo = ct.create_spin_half_xxz_mpo(ctx, 8, 1.0)
    W = mpo.sites[3]
    g = torch.Generator(device="cpu").manual_seed(9)
    dev = ctx.torch_device

    def sym(t):
        return (0.5 * (t + t.transpose(1, 2))).contiguous()

    th = ct.DenseTensor(torch.randn(chi * 4 * chi, generator=g, dtype=torch.float64).to(dev), [chi, 2, 2, chi])
    Le = ct.DenseTensor(sym(torch.randn(MPO_D, chi, chi, generator=g, dtype=torch.float64)).reshape(-1).to(dev),
                        [MPO_D, chi, chi])
    Re = ct.DenseTensor(sym(torch.randn(MPO_D, chi, chi, generator=g, dtype=torch.float64)).reshape(-1).to(dev),
                        [MPO_D, chi, chi])

    def run():
        return ct.lanczos_two_site_optimize(th, Le, Re, W, W, ctx, max_iter=LANCZOS, tol=1e-10, prec=args.prec,
                                            max_rotations=0, reorth=True)

    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    ctx.call("ct_kernel_timing", 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = _lib.launch_count()
    e0.record()
    for _ in range(args.steps):
        E, _ = run()
    e1.record()
    torch.cuda.synchronize()
    launches = _lib.launch_count() - n0

    def read_class(cls):
        n_kt, ms_kt, fl_kt = C.c_int64(), C.c_double(), C.c_double()
        ctx.call("ct_kernel_timing_read_class", cls, C.byref(n_kt), C.byref(ms_kt), C.byref(fl_kt))
        return n_kt.value, ms_kt.value * 1e-3, fl_kt.value

    _, heff_s, _ = read_class(1)
    nvec, vec_s, vec_bytes = read_class(3)
    ctx.call("ct_kernel_timing", 0)
    s = e0.elapsed_time(e1) * 1e-3 / max(args.steps, 1)
    peaks = read_peaks()
    print(json.dumps({"metric": "Lanczos run seconds", "value": s, "unit": "s/run", "dtype": args.prec,
                      "config": {"workload": f"centre-bond Lanczos chi={chi} D=5 d=2, {LANCZOS} steps, "
                                             "reorthogonalised"},
                      "energy": E, "heff_s_per_run": heff_s / max(args.steps, 1),
                      "vector_s_per_run": vec_s / max(args.steps, 1), "vector_steps": nvec,
                      "vector_bytes_per_run": vec_bytes / max(args.steps, 1),
                      "lanczos_gbs": vec_bytes / max(vec_s, 1e-12) / 1e9,
                      "lanczos_frac_of_hbm": vec_bytes / max(vec_s, 1e-12) / 1e9 / peaks.get("hbm_gbs", 6800.0),
                      "steps": args.steps, "warmup": args.warmup, "gpu_launches": launches}), flush=True)


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def split_mode(args):
    """W + K warm subspace splits (ct_svd_split_warm) of a chi=1024 centre bond (profiling workload).

    theta [1024, 2, 2, 1024] with singular values exp(-0.012 k) and random
    singular vectors; the start basis is the exact right basis perturbed by
    1e-5 noise and re-orthonormalised, i.e. a basis kept by the previous
    visit of the bond.  One JSON line.
    """
    import ctypes as C
    import torch
    import chemtensor_mojo_gb300 as ct
    ctx = ct.get_context(0)
    dev = ctx.torch_device
    Dl = Dr = args.chi
    d = D_PHYS
    m = n = Dl * d
    c = args.chi
    g = np.random.default_rng(4)
    U, _ = np.linalg.qr(g.standard_normal((m, m)))
    V, _ = np.linalg.qr(g.standard_normal((n, n)))
    s = np.exp(-0.012 * np.arange(m))
    M = (U * s) @ V.T
    X, _ = np.linalg.qr((V[:, :c] + 1e-5 * g.standard_normal((n, c))))
    th = torch.from_numpy(M.reshape(Dl, d, d, Dr).copy()).to(dev)
    Xd = torch.from_numpy(np.ascontiguousarray(X.T)).to(dev)
    bout = torch.empty(c * m, dtype=torch.float64, device=dev)
    A = torch.empty(m * c, dtype=torch.float64, device=dev)
    B = torch.empty(c * n, dtype=torch.float64, device=dev)
    acc, disc = C.c_int(), C.c_double()

    def one():
        ctx.call("ct_svd_split_warm", C.c_void_p(th.data_ptr()), Dl, d, Dr, c, 1, C.c_void_p(Xd.data_ptr()), 0,
                 C.c_void_p(bout.data_ptr()), C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()), C.byref(acc),
                 C.byref(disc), None)

    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one()
    torch.cuda.synchronize()
    sec = (time.perf_counter() - t0) / max(args.steps, 1)
    opt = float(np.sum(s[c:] ** 2) / np.sum(s ** 2))
    print(json.dumps({"metric": "warm subspace split seconds", "value": sec, "unit": "s/split",
                      "config": {"workload": f"theta {m}x{n}, chi={c}, left-to-right, no power steps"},
                      "accepted": acc.value, "discarded": disc.value, "optimal_discarded": opt,
                      "steps": args.steps, "warmup": args.warmup}), flush=True)


def hubbard_mode(args):
    """Large mixed-precision run with gradient, at the chi this box's time allows.

    1D Fermi-Hubbard chain (Jordan-Wigner), L=48, d=4, t=1, U=8, MPO bond
    dimension 6; seeded Gaussian initial MPS; chi_max ramped 256 -> 512 ->
    1024 (two sweeps each) or, with --chi 2048, 256 -> 512 -> 1024 -> 2048
    over ten sweeps (2, 2, 3, 3), 24 Lanczos steps, eps_trunc = 0, in the mixed
    form with kept bases across the ramp and randomized first-visit splits (two
    power steps); then one adjoint-gradient pass at the final state in the
    mixed form (environment checkpoints every 7 sites).  Reports sweep seconds per chi,
    the FP64 Rayleigh energy, the gradient residual |grad E| (zero at a
    stationary state), |dE/E| of the mixed form against the FP64 form after two
    sweeps at chi=256 and two more at 512 (same start, Jacobi first visits in
    both) and peak device memory.  One JSON line.
    """
    import ctypes as C
    import torch
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300 import _lib
    from chemtensor_mojo_gb300.autograd import energy_and_gradient
    ctx = ct.get_context(0)
    L = 48
    if args.chi >= 2048:
        ramp, nsw = [256, 512, 1024, 2048], [2, 2, 3, 3]
    else:
        ramp = [256, 512, 1024] if args.chi >= 1024 else [c for c in (256, 512, 1024) if c <= args.chi]
        nsw = [2] * len(ramp)
    if args.ramp_sweeps:
        nsw = [int(x) for x in args.ramp_sweeps.split(",")][:len(ramp)]
        ramp = ramp[:len(nsw)]
    mpo = ct.create_fermi_hubbard_mpo(ctx, L, 1.0, 8.0)
    arrays, _ = ct.random_mps_c_compatible_arrays(L, 4, ramp[0], 11)
    mps = ct.mps_right_normalize(ctx, ct.mps_from_arrays(ctx, arrays))
    free0, total = torch.cuda.mem_get_info()
    peak_used = 0
    log = []
    first = True
    for chi, ns in zip(ramp, nsw):
        st = ct.DMRGStats()
        p = ct.DMRGParams(num_sweeps=ns, chi_max=chi, eps_trunc=0.0, max_krylov_iter=LANCZOS, krylov_tol=1e-10,
                          energy_tol=0.0, max_rotations=0, prec="tf32x3", final_rayleigh=True,
                          keep_bases=not first, cold_power_steps=2, verbose=2 if args.verbose else 0)
        E, mps = ct.dmrg_two_site(ctx, mpo, mps, p, st)
        first = False
        free, _ = torch.cuda.mem_get_info()
        peak_used = max(peak_used, total - free)
        log.append({"chi_max": chi, "sweeps": ns,
                    "seconds_per_sweep": (st.seconds_total - st.seconds_rayleigh) / ns,
                    "seconds_final_rayleigh_fp64": st.seconds_rayleigh, "completed_rows": st.completed_rows,
                    "sweep_energies": st.sweep_energies, "energy_rayleigh": st.energy_rayleigh,
                    "subspace_splits": st.subspace_splits, "cold_splits": st.cold_splits,
                    "exact_splits": st.exact_splits, "heff_tflops": st.heff_flops / max(st.seconds_lanczos, 1e-12) / 1e12,
                    "seconds": {"lanczos": st.seconds_lanczos, "split": st.seconds_svd,
                                "split_subspace": st.seconds_subspace, "env": st.seconds_env},
                    "max_discarded": st.max_discarded})
    accuracy, gradient = None, None
    if not args.no_extras:
        # mixed vs FP64 form on the same start: two sweeps at chi=256, then two at 512
        # (Jacobi first visits in both forms, so the difference is precision, not the start);
        # FP64 Rayleigh energy after each call in both forms
        stages = [c for c in (256, 512) if c <= max(ramp)]
        acc_e = {}
        acc_t = {}
        for pr in ("fp64", "tf32x3"):
            mps_c = ct.mps_right_normalize(ctx, ct.mps_from_arrays(ctx, arrays))
            acc_e[pr], acc_t[pr] = [], []
            for k, c in enumerate(stages):
                st_c = ct.DMRGStats()
                _, mps_c = ct.dmrg_two_site(ctx, mpo, mps_c, ct.DMRGParams(
                    num_sweeps=2, chi_max=c, eps_trunc=0.0, max_krylov_iter=LANCZOS, krylov_tol=1e-10,
                    energy_tol=0.0, max_rotations=0, prec=pr, final_rayleigh=True,
                    keep_bases=(pr == "tf32x3" and k > 0)), st_c)
                acc_e[pr].append(st_c.energy_rayleigh)
                acc_t[pr].append((st_c.seconds_total - st_c.seconds_rayleigh) / 2)
        accuracy = {"chi_max_stages": stages, "sweeps_per_stage": 2, "E_fp64": acc_e["fp64"],
                    "E_mixed_rayleigh_fp64": acc_e["tf32x3"],
                    "dE_over_E": [abs(a - b) / abs(b) for a, b in zip(acc_e["tf32x3"], acc_e["fp64"])],
                    "seconds_per_sweep": acc_t,
                    "note": "FP64 Rayleigh energies of both forms after each stage, same start"}
        sites = [s.tensor.storage[: int(np.prod(s.tensor.shape))].view(*s.tensor.shape) for s in mps.sites]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Eg, grads = energy_and_gradient(mpo, sites, checkpoint_every=7, ctx=ctx, prec="tf32x3")
        torch.cuda.synchronize()
        tg = time.perf_counter() - t0
        free, _ = torch.cuda.mem_get_info()
        peak_used = max(peak_used, total - free)
        gnorm = float(torch.sqrt(sum((g * g).sum() for g in grads)))
        gradient = {"energy": Eg, "seconds": tg, "norm": gnorm, "checkpoint_every": 7, "dtype": "tf32x3"}
    print(json.dumps({"metric": "Fermi-Hubbard L=48 mixed sweep seconds", "unit": "s/sweep", "data": "synthetic",
                      "config": {"workload": "1D Fermi-Hubbard JW L=48 d=4 t=1 U=8 D=6, chi ramp " +
                                 "->".join(str(c) for c in ramp) + " (sweeps " + "+".join(str(n) for n in nsw) +
                                 "), lanczos=24, eps=0"},
                      "ramp": log, "accuracy_vs_fp64": accuracy,
                      "gradient": gradient,
                      "peak_device_bytes": int(peak_used), "device_bytes_before": int(total - free0)}),
          flush=True)


ACC_SEED = 7


def schedule_run(ctx, ct, mpo, arrays, schedule, prec):
    """One call of dmrg_two_site per sweep of `schedule` (chi_max per sweep) from the
    right-normalised MPS of `arrays`; the FP64 Rayleigh quotient of the MPS after each
    sweep, contracted on the device.  Per sweep: chi_max, Lanczos energy, Rayleigh
    energy, seconds (the call's wall clock without the Rayleigh contraction), splits."""
    mps = ct.mps_right_normalize(ctx, ct.mps_from_arrays(ctx, arrays))
    out = []
    st = None
    for k, c in enumerate(schedule):
        st = ct.DMRGStats()
        E, mps = ct.dmrg_two_site(ctx, mpo, mps, ct.DMRGParams(
            num_sweeps=1, chi_max=c, eps_trunc=EPS, max_krylov_iter=LANCZOS, krylov_tol=1e-10, energy_tol=0.0,
            max_rotations=0, prec=prec, final_rayleigh=True, keep_bases=(prec == "tf32x3" and k > 0)), st)
        out.append({"chi_max": c, "energy_lanczos": E, "energy_rayleigh": st.energy_rayleigh,
                    "seconds": st.seconds_total - st.seconds_rayleigh, "seconds_rayleigh": st.seconds_rayleigh,
                    "seconds_lanczos": st.seconds_lanczos, "seconds_split": st.seconds_svd,
                    "seconds_env": st.seconds_env, "max_discarded": st.max_discarded,
                    "subspace_splits": st.subspace_splits, "exact_splits": st.exact_splits})
    return out, mps, list(st.discarded)


def fp64_ref_mode(args):
    """The plain FP64 form against the mixed form at the headline size.

    Heisenberg chain L=64 (D=5, d=2), seeded Gaussian start (seed 7), right-
    normalised; chi_max 64, 256, then --steps sweeps at --chi (1024), one call
    per sweep, 24 Lanczos steps, eps_trunc = 0, converged eigensolve, in both
    forms.  Reports each form's seconds per sweep at --chi (measured, not
    estimated) and, per sweep, |dE/E| between the FP64 Rayleigh quotients of the
    two forms' MPS.  The FP64 form's trajectory is deterministic (fixed-order
    reductions), so its energies serve later runs of the mixed form on the same
    schedule as the reference (--out writes the JSON line to a file).
    """
    import chemtensor_mojo_gb300 as ct
    ctx = ct.get_context(0)
    L = args.L
    mpo = ct.create_spin_half_xxz_mpo(ctx, L, 1.0)
    arrays, _ = ct.random_mps_c_compatible_arrays(L, D_PHYS, RAMP[0], ACC_SEED)
    schedule = [64, 256] + [args.chi] * max(args.steps, 1)
    runs, states, disc = {}, {}, {}
    for pr in args.forms.split(","):
        runs[pr], states[pr], disc[pr] = schedule_run(ctx, ct, mpo, arrays, schedule, pr)
    line = {"metric": "FP64 vs mixed two-site sweep at chi_max", "unit": "s/sweep", "data": "synthetic",
            "config": {"workload": f"heisenberg_xxz L={L} d=2 D=5 seed={ACC_SEED} chi schedule "
                                   f"{','.join(map(str, schedule))} lanczos={LANCZOS} eps={EPS}",
                       "eigensolver": "converged tridiagonal"},
            "schedule": schedule, "runs": runs}
    at = [k for k, c in enumerate(schedule) if c == args.chi]
    for pr, r in runs.items():
        # the first sweep at chi grows the bonds; the last one is the steady state
        line[f"{pr}_s_per_sweep_at_chi"] = float(np.mean([r[k]["seconds"] for k in at]))
        line[f"{pr}_s_last_sweep"] = float(r[-1]["seconds"])
    if "fp64" in runs and "tf32x3" in runs:
        a, b = runs["tf32x3"], runs["fp64"]
        line["dE_over_E_each_sweep"] = [abs(x["energy_rayleigh"] - y["energy_rayleigh"]) / abs(y["energy_rayleigh"])
                                        for x, y in zip(a, b)]
        line["dE_over_E_at_chi"] = max(line["dE_over_E_each_sweep"][k] for k in at)
        line["speedup_mixed_vs_fp64_at_chi"] = line["fp64_s_per_sweep_at_chi"] / line["tf32x3_s_per_sweep_at_chi"]
        line["speedup_mixed_vs_fp64_last_sweep"] = line["fp64_s_last_sweep"] / line["tf32x3_s_last_sweep"]
        # Schmidt spectra of every bond of the two final states (FP64 device SVD) and the
        # discarded weights of the last sweep's 2(L-1) splits
        sa, sb = ct.mps_schmidt_values(states["tf32x3"], ctx), ct.mps_schmidt_values(states["fp64"], ctx)
        w_err, top_rel = 0.0, 0.0
        for x, y in zip(sa, sb):
            n = min(len(x), len(y))
            w_err = max(w_err, float(np.max(np.abs(x[:n] ** 2 - y[:n] ** 2))))   # weights of a normalised state
            top_rel = max(top_rel, float(np.max(np.abs(x[:8] - y[:8]) / y[:8])))
        da, db = np.array(disc["tf32x3"]), np.array(disc["fp64"])
        line["spectrum_check"] = {
            "bonds": len(sa), "max_abs_weight_diff": w_err, "max_rel_diff_top8_schmidt_values": top_rel,
            "last_sweep_discarded_max_abs_diff": float(np.max(np.abs(da - db))) if len(da) == len(db) else None,
            "last_sweep_discarded_max": {"tf32x3": float(da.max()), "fp64": float(db.max())},
            "note": "final MPS of each form; weights s^2 of the normalised state at every bond"}
    print(json.dumps(line), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            f.write(json.dumps(line) + "\n")


def heff_grid_mode(args):
    """Kernel grid: chi in {256, 512, 1024, 2048} x D in {5, 16, 32} x d in {2, 4}.

    Random L, R [D, chi, chi], W [D, d, d, D] symmetrised in (s, t), theta
    [chi, d, d, chi] and a site A [chi, d, chi], all N(0, 1) from a fixed seed.
    Each point: one H_eff apply and one left-environment update, each with one
    warm-up and ``--steps`` timed calls (CUDA events), in the TF32x3 form and,
    where one apply stays under ~2 s (algorithmic FLOPs <= 2.5 TFLOP), in the
    FP64 form.  FLOPs: H_eff 4 D d^2 chi^3 + 4 D^2 d^3 chi^2, environment
    4 D d chi^3 + 2 D^2 d^2 chi^2.  One JSON line.
    """
    import torch
    import chemtensor_mojo_gb300 as ct
    ctx = ct.get_context(0)
    dev = ctx.torch_device
    g = torch.Generator(device="cpu").manual_seed(11)
    rows = []
    for chi in (256, 512, 1024, 2048):
        for D in (5, 16, 32):
            for d in (2, 4):
                F = heff_flops(chi, chi, D, d)
                w = torch.randn(D, d, d, D, generator=g, dtype=torch.float64)
                w = 0.5 * (w + w.transpose(1, 2))
                mpo = ct.mpo_from_arrays(ctx, [w.numpy(), w.numpy()])
                th = ct.DenseTensor(torch.randn(chi * d * d * chi, generator=g, dtype=torch.float64).to(dev),
                                    [chi, d, d, chi])
                Le = ct.DenseTensor(torch.randn(D * chi * chi, generator=g, dtype=torch.float64).to(dev),
                                    [D, chi, chi])
                Re = ct.DenseTensor(torch.randn(D * chi * chi, generator=g, dtype=torch.float64).to(dev),
                                    [D, chi, chi])
                A = ct.MPSSite(ct.DenseTensor(torch.randn(chi * d * chi, generator=g, dtype=torch.float64).to(dev),
                                              [chi, d, chi]))
                Fe = 4.0 * D * d * chi ** 3 + 2.0 * D * D * d * d * chi ** 2
                row = {"chi": chi, "D": D, "d": d, "heff_gflop": F / 1e9, "env_gflop": Fe / 1e9}

                def timed(fn):
                    fn()
                    torch.cuda.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    for _ in range(max(args.steps, 1)):
                        fn()
                    e1.record()
                    torch.cuda.synchronize()
                    return e0.elapsed_time(e1) * 1e-3 / max(args.steps, 1)

                for prec in ("tf32x3", "fp64"):
                    if prec == "fp64" and F > 2.5e12:
                        continue
                    sec = timed(lambda: ct.apply_two_site_heff(th, Le, Re, mpo.sites[0], mpo.sites[1], ctx,
                                                               prec=prec))
                    sec_e = timed(lambda: ct.update_left_environment(Le, A, mpo.sites[0], ctx, prec))
                    row[prec] = {"heff_s": sec, "heff_tflops": F / sec / 1e12, "env_s": sec_e,
                                 "env_tflops": Fe / sec_e / 1e12}
                rows.append(row)
                print(json.dumps(row), file=sys.stderr, flush=True)
                del th, Le, Re, mpo, A
                torch.cuda.empty_cache()
    print(json.dumps({"metric": "H_eff apply and left-environment update TFLOP/s (kernel grid)", "unit": "TFLOP/s",
                      "data": "synthetic", "steps": args.steps,
                      "config": {"workload": "chi x D x d grid, random L/R/W/theta/A, N(0,1) seed 11"},
                      "grid": rows}), flush=True)


# ---------------------------------------------------------------------------
def contractions_mode(args):
    """The contraction operations of bench_contractions.mojo:349-475 on the same inputs
    (Ising MPO J=1, h=g=0; C-compatible random MPS with seeds 42 and 43 at
    (nsites, d, chi)), timed with CUDA events: <chi|W|psi> (sign flipped to the C
    convention), W|psi> (result ||W psi||), <chi|psi>, and the left-environment
    sweep.  One JSONL record per operation in the reference's record format, and
    one summary JSON line."""
    import torch
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300 import environments as ct_env
    ctx = ct.get_context(0)
    n, d, chi, runs = args.nsites, args.d, args.chi, max(args.runs, 1)
    mpo = ct.create_ising_1d_mpo(ctx, n, J=1.0, h_longitudinal=0.0, g_transverse=0.0)
    if d != 2:
        raise SystemExit("contractions: the Ising MPO has d = 2")
    psi = ct.create_random_mps_c_compatible(ctx, n, d, chi, 42)
    phi = ct.create_random_mps_c_compatible(ctx, n, d, chi, 43)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(runs):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / runs

    def left_env_sweep():
        L = ct_env.create_identity_environment(ctx, mpo.bond_dimension(0), psi.bond_dimension(0))
        for i in range(n):
            L = ct.update_left_environment(L, psi.sites[i], mpo.sites[i], ctx)
        return L

    recs = []
    t = timed(lambda: ct.expectation_value_two_mps(phi, mpo, psi, ctx))
    recs.append(("mps_mpo_inner", t, -ct.expectation_value_two_mps(phi, mpo, psi, ctx)))
    t = timed(lambda: ct.apply_mpo(mpo, psi, ctx))
    op_psi = ct.apply_mpo(mpo, psi, ctx)
    recs.append(("mps_mpo_apply", t, math.sqrt(max(ct.mps_overlap(op_psi, op_psi, ctx), 0.0))))
    t = timed(lambda: ct.mps_overlap(phi, psi, ctx))
    recs.append(("mps_mps", t, ct.mps_overlap(phi, psi, ctx)))
    t = timed(left_env_sweep)
    recs.append(("left_env_sweep", t, 0.0))
    for op, t, res in recs:
        line = json.dumps({"backend": "gb300", "operation": op, "params": {"nsites": n, "d": d, "chi_max": chi},
                           "time_seconds": t, "result": res, "runs": runs}, separators=(",", ":"))
        if args.jsonl:
            with open(args.jsonl, "a") as f:
                f.write(line + "\n")
        print(line, file=sys.stderr)
    print(json.dumps({"metric": "MPS/MPO contraction seconds", "unit": "s/op", "dtype": "fp64",
                      "config": {"workload": f"Ising MPO, C-compatible random MPS seeds 42/43, nsites={n} d={d} "
                                             f"chi_max={chi}"},
                      "ops": {op: {"seconds": t, "result": res} for op, t, res in recs}, "runs": runs}))


def heff_flops(chi_l, chi_r, D=MPO_D, d=D_PHYS):
    return (2.0 * chi_l * D * d * d * chi_r * chi_l + 2.0 * chi_l * d * chi_r * D * d * d * D
            + 2.0 * chi_l * chi_r * d * D * d * d * D + 2.0 * chi_l * d * d * chi_r * D * chi_r)


def bond_caps(L, chi):
    return [min(chi, 2 ** k, 2 ** (L - k)) for k in range(L + 1)]


def sweep_flop_weight(L, chi):
    """sum over the 2(L-1) local updates of H_eff FLOPs relative to the centre bond."""
    c = bond_caps(L, chi)
    centre = heff_flops(chi, chi)
    w = sum(heff_flops(c[i], c[i + 2]) for i in range(L - 1))
    return 2.0 * w / centre


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)

    def summary(self):
        sm = []
        mx = []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def cpu_local_update_seconds(chi, seed=0):
    """One centre-bond local update of the CPU FP64 oracle (theta, Lanczos, SVD, env)."""
    from oracle import dmrg as od
    from oracle import hamiltonians as oh
    g = np.random.default_rng(seed)
    mpo = oh.spin_half_xxz(8, 1.0)
    W = mpo[3]
    A = g.standard_normal((chi, D_PHYS, chi)) / np.sqrt(2 * chi * chi)
    B = g.standard_normal((chi, D_PHYS, chi)) / np.sqrt(2 * chi * chi)
    Lenv = g.standard_normal((MPO_D, chi, chi))
    Lenv = 0.5 * (Lenv + Lenv.transpose(0, 2, 1))
    Renv = g.standard_normal((MPO_D, chi, chi))
    Renv = 0.5 * (Renv + Renv.transpose(0, 2, 1))
    t0 = time.perf_counter()
    th = od.build_two_site_theta(A, B)
    E, tho = od.lanczos_two_site_optimize(th, Lenv, Renv, W, W, LANCZOS, 1e-10, eig="exact")
    An, Bn, info = od.split_two_site_theta_svd(tho, chi, EPS, True)
    od.update_left_environment(Lenv, An, W)
    return time.perf_counter() - t0


def cpu_threads() -> int:
    """Threads the oracle's BLAS runs with: the pinned count when one is set, else every core."""
    for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        v = os.environ.get(var)
        if v and v.isdigit() and int(v) > 0:
            return int(v)
    return os.cpu_count() or 1


def cpu_sweep_seconds(L, chi, seed=3):
    """One full sweep of the CPU FP64 oracle (converged eigensolve, eps_trunc = 0) on the
    Heisenberg chain at chi_max = chi, from the seeded random MPS right-normalised with
    bond dimensions min(2^k, 2^(L-k), chi): every bond runs at its full size."""
    from oracle import dmrg as od
    from oracle import hamiltonians as oh
    from oracle import rng as orng
    mpo = oh.spin_half_xxz(L, 1.0)
    sites, _ = orng.create_random_mps_c_compatible(L, D_PHYS, chi, seed)
    mps = od.right_normalize(sites)
    t0 = time.perf_counter()
    od.dmrg_two_site(mpo, mps, od.DMRGParams(1, chi, EPS, LANCZOS, 1e-10, 0.0), eig="exact")
    return time.perf_counter() - t0


def reference_arm(args, rank):
    """CPU oracle port of the reference path: sampled centre-bond updates, extrapolated.

    The extrapolation (centre-bond local update x the sweep's FLOP weight) is checked
    once per run at chi = 256, where a whole CPU sweep is affordable: the measured
    sweep and its extrapolation are both reported."""
    if rank != 0:
        return
    chi = args.chi
    for _ in range(args.warmup):
        cpu_local_update_seconds(min(chi, 256))
    times = [cpu_local_update_seconds(chi, seed=s) for s in range(args.steps)]
    weight = sweep_flop_weight(args.L, chi)
    per_sweep = float(np.mean(times)) * weight
    chk = min(chi, 256)
    t_centre = float(np.mean([cpu_local_update_seconds(chk, seed=s) for s in range(3)]))
    t_sweep = cpu_sweep_seconds(args.L, chk)
    extrapolated = t_centre * sweep_flop_weight(args.L, chk)
    check = {"chi_max": chk, "measured_sweep_s": t_sweep, "extrapolated_sweep_s": extrapolated,
             "measured_over_extrapolated": t_sweep / extrapolated,
             "note": "one whole CPU sweep vs 3 centre-bond local updates x the FLOP weight"}
    line = {
        "impl": "reference", "metric": METRIC, "value": per_sweep, "unit": "s/sweep", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_sweep * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"heisenberg_xxz L={args.L} d=2 D=5 chi={chi} lanczos={LANCZOS}",
                   "model": "spin-1/2 XXZ Delta=1 (reference XXZ MPO, J=-1/4)", "parallelism": "replicas"},
        "cpu_baseline": {"value": per_sweep, "unit": "s/sweep", "cores": cpu_threads(), "kind": "port",
                         "sample": f"{args.steps} centre-bond local updates at chi={chi}, FLOP-weighted x{weight:.1f}"
                                   " to a sweep (extrapolated)"},
        "e2e": {"value": per_sweep, "unit": "s/sweep", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_extrapolation_check": check,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def replica_max(dist, *seconds):
    """Max over ranks of each timing (replicas: no collective on the data path,
    only this reduction of the timed region's clocks, over gloo)."""
    if dist is None:
        return seconds
    import torch
    t = torch.tensor(list(seconds), dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return tuple(float(x) for x in t)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank)
        return
    if args.mode == "contractions":
        return contractions_mode(args)
    if args.mode == "split":
        split_mode(args)
        return
    if args.mode == "hubbard":
        hubbard_mode(args)
        return
    if args.mode == "heff-grid":
        heff_grid_mode(args)
        return
    if args.mode == "fp64-ref":
        fp64_ref_mode(args)
        return
    if args.mode == "lanczos":
        lanczos_mode(args)
        return
    if args.mode == "fp64tc":
        fp64tc_mode(args)
        return
    if args.mode == "heff":
        heff_mode(args)
        return

    import torch
    import ctypes as C
    import chemtensor_mojo_gb300 as ct
    from chemtensor_mojo_gb300 import _lib
    from chemtensor_mojo_gb300.dmrg import bond_capacities

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    ctx = ct.get_context(local_rank)
    L = args.L
    chi = args.chi
    prec = args.prec

    mpo = ct.create_spin_half_xxz_mpo(ctx, L, 1.0)
    arrays, dims = ct.random_mps_c_compatible_arrays(L, D_PHYS, RAMP[0], 1000 + rank)
    mps = ct.mps_right_normalize(ctx, ct.mps_from_arrays(ctx, arrays))

    def params(c, nsweeps, pr=prec):
        return ct.DMRGParams(num_sweeps=nsweeps, chi_max=c, eps_trunc=EPS, max_krylov_iter=LANCZOS,
                             krylov_tol=1e-10, energy_tol=0.0, max_rotations=0, prec=pr)

    # ---- warm-up: the chi ramp ----------------------------------------------
    ramp = (RAMP + [chi] * 100)[:max(args.warmup, 0)]
    ramp = [min(c, chi) for c in ramp]
    E = None
    warm_log = []
    for c in ramp:
        st = ct.DMRGStats()
        E, mps = ct.dmrg_two_site(ctx, mpo, mps, params(c, 1), st)
        warm_log.append({"chi_max": c, "energy": E, "seconds": st.seconds_total})

    # ---- timed: K sweeps at chi, from pinned host buffers --------------------
    d = D_PHYS
    cap = bond_capacities(list(mps.bond_dims), d, chi)
    host_sites = [torch.zeros(cap[i] * d * cap[i + 1], dtype=torch.float64).pin_memory() for i in range(L)]
    for i, s in enumerate(mps.sites):
        host_sites[i][:s.tensor.size].copy_(s.tensor.storage.cpu())
    host_mpo = [s.tensor.storage.cpu().pin_memory() for s in mpo.sites]
    dev_sites = [torch.empty_like(h, device=ctx.torch_device) for h in host_sites]
    dev_mpo = [torch.empty_like(h, device=ctx.torch_device) for h in host_mpo]
    bd = _lib.i64_array(mps.bond_dims)
    mpo_pp, k1 = _lib.ptr_array([t.data_ptr() for t in dev_mpo])
    mps_pp, k2 = _lib.ptr_array([t.data_ptr() for t in dev_sites])
    capacity = _lib.i64_array([t.numel() for t in dev_sites])
    Ec = C.c_double()
    sweeps_e = (C.c_double * max(args.steps, 1))()
    done = C.c_int()
    stats = _lib.ct_dmrg_stats()
    # the timed sweeps continue the warm-up's MPS on the same handle, so the
    # large splits of the first half-sweep start from the kept bond bases
    tp = params(chi, args.steps)
    tp.keep_bases = True
    # the reported energy is the FP64 Rayleigh quotient of the final MPS, contracted
    # on the device inside the timed call (its cost is part of `value`)
    tp.final_rayleigh = True
    tp.verbose = 2 if args.verbose else 0
    cp = tp.to_c()
    h2d = sum(h.numel() * 8 for h in host_sites) + sum(h.numel() * 8 for h in host_mpo)
    d2h = sum(h.numel() * 8 for h in host_sites) + 8

    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    clocks = ClockSampler(local_rank)
    # event pair around every tensor-core GEMM launch of the timed sweeps
    kt_on = prec == "tf32x3"
    if kt_on:
        ctx.call("ct_kernel_timing", 1)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches0 = _lib.launch_count()
    t_wall0 = time.perf_counter()
    ev[0].record(stream)
    for h, dv in zip(host_sites, dev_sites):
        dv.copy_(h, non_blocking=True)
    for h, dv in zip(host_mpo, dev_mpo):
        dv.copy_(h, non_blocking=True)
    ev[1].record(stream)
    ctx.call("ct_dmrg_two_site", C.byref(cp), L, d, _lib.i64_array(mpo.bond_dims), mpo_pp, bd, mps_pp, capacity,
             C.byref(Ec), sweeps_e, C.byref(done), None, C.byref(stats))
    ev[2].record(stream)
    for h, dv in zip(host_sites, dev_sites):
        h.copy_(dv, non_blocking=True)
    ev[3].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    launches = _lib.launch_count() - launches0
    clocks.stop()
    kt = None
    kt_heff = None
    kt_centre = None
    kt_vec = None
    if kt_on:
        def read_class(cls):
            n_kt, ms_kt, fl_kt = C.c_int64(), C.c_double(), C.c_double()
            ctx.call("ct_kernel_timing_read_class", cls, C.byref(n_kt), C.byref(ms_kt), C.byref(fl_kt))
            return {"launches": n_kt.value, "ms": ms_kt.value, "flops": fl_kt.value}
        kt = read_class(0)        # every TF32x3 GEMM launch
        kt_heff = read_class(1)   # every whole H_eff apply inside Lanczos
        kt_centre = read_class(2)  # the applies at the largest size (centre bonds at chi_max)
        kt_vec = read_class(3)     # Krylov vector work of every Lanczos step (flops field: bytes)
        ctx.call("ct_kernel_timing", 0)
    if dist is not None:
        dist.barrier()
    K = max(args.steps, 1)
    dev_s = ev[1].elapsed_time(ev[2]) * 1e-3
    e2e_s = ev[0].elapsed_time(ev[3]) * 1e-3
    dev_s, e2e_s = replica_max(dist, dev_s, e2e_s)
    # whole job: every rank ran K sweeps of its own replica in the max-over-ranks time
    per_sweep = dev_s / (K * world)
    heff_tflops = stats.heff_flops / max(stats.seconds_lanczos, 1e-12) / 1e12
    final_dims = [int(x) for x in bd]
    energy_rq = stats.energy_rayleigh

    extras = {}
    if rank == 0 and not args.no_extras:
        extras = side_measurements(ctx, ct, _lib, C, chi, prec, L, mpo)

    if rank != 0:
        return
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        peaks = {}
    bf16 = peaks.get("bf16_tflops", 1900.0)
    peak_src = "measured" if "bf16_tflops" in peaks else "fallback"
    line = {
        "metric": METRIC, "value": per_sweep, "unit": "s/sweep", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_sweep * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": prec, "storage_dtype": "f64", "data": "synthetic",
        "config": {"workload": f"heisenberg_xxz L={L} d=2 D=5 chi_max={chi} (ramp {ramp}) lanczos={LANCZOS} "
                               f"eps={EPS}", "model": "spin-1/2 XXZ Delta=1 (reference XXZ MPO, J=-1/4)",
                   "global_batch": 1, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (MPS + environments + Krylov basis >> 129 MB)",
                   "eigensolver": "converged tridiagonal Jacobi"},
        "energy": energy_rq, "energy_note": "FP64 Rayleigh quotient of the final MPS, inside the timed call",
        "seconds_final_rayleigh": stats.seconds_rayleigh, "energy_lanczos": Ec.value, "sweep_energies_lanczos": list(sweeps_e)[:done.value],
        "bond_dims_final": final_dims,
        "heff_tflops": heff_tflops, "heff_applies": stats.heff_applies, "local_updates": stats.local_updates,
        "phase_seconds": {"lanczos": stats.seconds_lanczos, "svd": stats.seconds_svd,
                          "svd_subspace": stats.seconds_subspace, "env": stats.seconds_env,
                          "total_wall": stats.seconds_total},
        "max_discarded": stats.max_discarded, "warmup_log": warm_log,
        "splits": {"subspace": stats.subspace_splits, "exact": stats.exact_splits},
        "e2e": {"value": e2e_s / (K * world), "unit": "s/sweep", "h2d_bytes_per_step": h2d // K,
                "d2h_bytes_per_step": d2h // K,
                "wall_s": t_wall},
        "gpu_launches": launches,
        "launches_before_timed": launches0,
        "clocks": clocks.summary(),
    }
    line.update(extras)
    if "fp64_sweep_s_estimate" in extras:
        line["speedup_vs_fp64_form_estimate"] = extras["fp64_sweep_s_estimate"] / per_sweep
    if kt and kt["launches"] > 0 and kt["ms"] > 0:
        # live: every TF32x3 GEMM launch of the timed sweeps, CUDA events on the launching stream
        ach = kt["flops"] / (kt["ms"] * 1e-3) / 1e12
        peak = bf16 / 6.0
        line["roofline"] = {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                            "traffic": TC_GEMM_TRAFFIC_BYTES,
                            "kernel": "tc_gemm_chunk_kernel<BN,STAGES> (TF32x3, tcgen05, a fresh TMEM accumulator "
                                      "every 64 of K summed in FP32 registers; tile width 128/192/224/256 and the "
                                      "transposed product chosen per shape, stream-K last wave)",
                            "launches": kt["launches"], "avg_launch_ms": kt["ms"] / kt["launches"],
                            "flops_per_launch": kt["flops"] / kt["launches"],
                            "share_of_timed_region": kt["ms"] * 1e-3 / max(dev_s, 1e-12),
                            "peak_note": f"{peak_src} bf16 {bf16} TFLOP/s / 2 (TF32 rate) / 3 (3 MMAs per product)",
                            "traffic_note": "DRAM read+write bytes of one centre-bond H_eff GEMM 1 "
                                            "(5120x4096x1024, tc_gemm_chunk_kernel<224,2>) from an ncu capture, "
                                            "per launch"}
    if kt_heff and kt_heff["launches"] > 0:
        # CUDA-event breakdown of the timed sweeps (device seconds, summed over both sweeps)
        heff_s = kt_heff["ms"] * 1e-3
        gemm_s = kt["ms"] * 1e-3 if kt else 0.0
        line["breakdown"] = {
            "timed_region_s": dev_s,
            "heff_apply_s": heff_s, "heff_apply_count": kt_heff["launches"],
            "heff_apply_tflops": kt_heff["flops"] / max(heff_s, 1e-12) / 1e12,
            "heff_apply_centre_count": kt_centre["launches"],
            "heff_apply_centre_ms": kt_centre["ms"] / max(kt_centre["launches"], 1),
            "heff_apply_centre_tflops": kt_centre["flops"] / max(kt_centre["ms"] * 1e-3, 1e-12) / 1e12,
            "heff_apply_centre_frac_of_3xtf32_peak": (kt_centre["flops"] / max(kt_centre["ms"] * 1e-3, 1e-12)
                                                      / 1e12) / (bf16 / 6.0),
            "tc_gemm_s_all": gemm_s,
            "lanczos_other_s": stats.seconds_lanczos - heff_s,
            "split_subspace_s": stats.seconds_subspace,
            "split_exact_s": stats.seconds_svd - stats.seconds_subspace,
            "env_s": stats.seconds_env,
            "note": "lanczos_other = Krylov vector kernels, eigensolve, Ritz vector; tc_gemm_s_all counts the "
                    "GEMMs of H_eff, environments and splits",
        }
    if kt_vec and kt_vec["launches"] > 0 and kt_vec["ms"] > 0:
        hbm = peaks.get("hbm_gbs", 6800.0)
        gbs = kt_vec["flops"] / (kt_vec["ms"] * 1e-3) / 1e9
        line["lanczos_vector"] = {
            "gbs": gbs, "frac_of_hbm": gbs / hbm, "hbm_peak_gbs": hbm,
            "peak_src": "measured" if "hbm_gbs" in peaks else "fallback",
            "seconds": kt_vec["ms"] * 1e-3, "steps": kt_vec["launches"], "bytes": kt_vec["flops"],
            "note": "every reorthogonalised Lanczos step of the timed sweeps: alpha (v_j, w read), recurrence "
                    "(w, v_j, v_{j-1} read, w written), Gram-Schmidt dots (w and j+1 basis vectors read), update "
                    "(read again, w written), next vector (w read, v written); 8 B per element, CUDA events on "
                    "the launching stream"}
    if "cpu_sweep_s" in extras:
        line["cpu_baseline"] = {"value": extras["cpu_sweep_s"], "unit": "s/sweep", "cores": cpu_threads(),
                                "kind": "port", "sample": extras["cpu_sample"]}
    print(json.dumps(line), flush=True)


def side_measurements(ctx, ct, _lib, C, chi, prec, L, mpo):
    import torch
    out = {}
    # dominant kernel: TF32x3 GEMM at the centre-bond H_eff shapes
    if prec == "tf32x3":
        m, n, k = MPO_D * chi, D_PHYS * D_PHYS * chi, chi
        ms = C.c_double()
        ctx.call("ct_tc_gemm_time", C.c_int64(m), C.c_int64(n), C.c_int64(k), 10, C.byref(ms))
        out["tc_gemm_ms"] = ms.value
        out["tc_gemm_shape"] = [m, n, k]
        m4, n4, k4 = chi * D_PHYS * D_PHYS, chi, MPO_D * chi
        ctx.call("ct_tc_gemm_time", C.c_int64(m4), C.c_int64(n4), C.c_int64(k4), 10, C.byref(ms))
        out["tc_gemm4_ms"] = ms.value
        out["tc_gemm4_shape"] = [m4, n4, k4]
    # H_eff apply at the centre bond: mixed and FP64
    g = torch.Generator(device="cpu").manual_seed(5)
    dev = ctx.torch_device
    th = ct.DenseTensor(torch.randn(chi * 4 * chi, generator=g, dtype=torch.float64).to(dev), [chi, 2, 2, chi])
    Le = ct.DenseTensor(torch.randn(MPO_D * chi * chi, generator=g, dtype=torch.float64).to(dev), [MPO_D, chi, chi])
    Re = ct.DenseTensor(torch.randn(MPO_D * chi * chi, generator=g, dtype=torch.float64).to(dev), [MPO_D, chi, chi])
    W = mpo.sites[L // 2]
    F = heff_flops(chi, chi)
    for pr, reps in (("tf32x3", 10), ("fp64", 2)):
        ct.apply_two_site_heff(th, Le, Re, W, W, ctx, prec=pr)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            o = ct.apply_two_site_heff(th, Le, Re, W, W, ctx, prec=pr)
        e1.record()
        torch.cuda.synchronize()
        s = e0.elapsed_time(e1) * 1e-3 / reps
        out[f"heff_apply_{pr}_s"] = s
        out[f"heff_apply_{pr}_tflops"] = F / s / 1e12
        if pr == "tf32x3":
            o_mixed = o.to_numpy()
        else:
            o64 = o.to_numpy()
    out["heff_apply_rel_err_tf32x3_vs_fp64"] = float(np.linalg.norm(o_mixed - o64) / np.linalg.norm(o64))
    out["heff_apply_speedup_vs_fp64"] = out["heff_apply_fp64_s"] / out["heff_apply_tf32x3_s"]
    # plain FP64 form of the sweep, estimated from its measured centre-bond pieces:
    # one FP64 Jacobi split of theta (2chi x 2chi) and the FP64 H_eff apply, weighted
    # like the sweep (H_eff by FLOPs; one full-size split per binding bond visit)
    thm = torch.randn(chi * 4 * chi, generator=g, dtype=torch.float64).to(dev)
    Ab = torch.empty(2 * chi * chi, dtype=torch.float64, device=dev)
    Bb = torch.empty(2 * chi * chi, dtype=torch.float64, device=dev)
    chi_c, disc_c = C.c_int64(), C.c_double()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.call("ct_svd_split", _lib.CT_PREC_FP64, C.c_void_p(thm.data_ptr()), chi, D_PHYS, chi, chi, 0.0, 1,
             C.c_void_p(Ab.data_ptr()), C.c_void_p(Bb.data_ptr()), None, C.byref(chi_c), C.byref(disc_c))
    torch.cuda.synchronize()
    split64 = time.perf_counter() - t0
    caps = bond_caps(L, chi)
    full_visits = 2 * sum(1 for i in range(L - 1) if min(2 * caps[i], 2 * caps[i + 2]) > chi)
    weight = sweep_flop_weight(L, chi)
    out["fp64_split_s"] = split64
    out["fp64_sweep_s_estimate"] = LANCZOS * out["heff_apply_fp64_s"] * weight + split64 * full_visits
    out["fp64_sweep_note"] = (f"{LANCZOS} FP64 H_eff applies x {weight:.1f} centre-bond FLOP weights + "
                              f"{full_visits} FP64 Jacobi splits of {2 * chi}x{2 * chi} (measured once)")
    # accuracy: mixed vs FP64 on the same ramp capped at chi=256 (FP64 affordable); the mixed
    # form continues each call from the previous one's kept bases, as in the timed sweeps
    arrays, _ = ct.random_mps_c_compatible_arrays(L, D_PHYS, RAMP[0], 7)
    res = {}
    per = {}
    tsec = {}
    for pr in ("tf32x3", "fp64"):
        mps = ct.mps_right_normalize(ctx, ct.mps_from_arrays(ctx, arrays))
        t0 = time.perf_counter()
        per[pr] = []
        for k, c in enumerate(ACC_RAMP):
            st = ct.DMRGStats()
            E, mps = ct.dmrg_two_site(ctx, mpo, mps, ct.DMRGParams(
                num_sweeps=1, chi_max=c, eps_trunc=EPS, max_krylov_iter=LANCZOS, krylov_tol=1e-10,
                energy_tol=0.0, max_rotations=0, prec=pr, final_rayleigh=(c == 256 and pr == "tf32x3"),
                keep_bases=(pr == "tf32x3" and k > 0)), st)
            if c == 256:
                per[pr].append(st.energy_rayleigh if pr == "tf32x3" else E)
        tsec[pr] = time.perf_counter() - t0
        res[pr] = per[pr][-1]
    rel = [abs(a - b) / abs(b) for a, b in zip(per["tf32x3"], per["fp64"])]
    out["accuracy_check"] = {"workload": f"same chain, chi ramp {','.join(map(str, ACC_RAMP))} ({L} sites)",
                             "E_fp64": res["fp64"],
                             "E_tf32x3_rayleigh_fp64": res["tf32x3"],
                             "dE_over_E": abs(res["tf32x3"] - res["fp64"]) / abs(res["fp64"]),
                             "dE_over_E_each_chi256_sweep": rel,
                             "seconds_fp64": tsec["fp64"], "seconds_tf32x3": tsec["tf32x3"]}
    # CPU baseline: one centre-bond local update of the FP64 oracle, extrapolated
    t_cpu = cpu_local_update_seconds(chi)
    w = sweep_flop_weight(L, chi)
    out["cpu_sweep_s"] = t_cpu * w
    out["cpu_sample"] = (f"1 centre-bond local update (theta, {LANCZOS} Lanczos H_eff applies, SVD, env) at chi={chi}"
                         f" took {t_cpu:.2f} s; x{w:.1f} FLOP weight to a sweep (extrapolated)")
    return out


if __name__ == "__main__":
    main()
