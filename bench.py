#!/usr/bin/env python
"""Benchmark of the CISD_SO hot path on one GB300.

Workload: synthetic spin-orbital CISD, o/v = 60/240 occupied/virtual spin
orbitals (nso = 300, naux = 1200 Hermitian factors, seed 0, diagonal Fock from
per-spatial-orbital energies).  A step is one mixed-precision CISD_SO
iteration at DIIS steady state: the residual of apyib/ci_wfn.py:309-334 with
every contraction as complex FP32 via 3xTF32 tcgen05 MMAs, the FP64 amplitude
update, the FP64 DIIS Gram row and the FP64 extrapolation + energy + norms.
The metric counts algorithmic work per residual,
W = 8 * (o^2 v^4 / 2 + o^3 v^3 + o^4 v^2 / 2 + 5 o^2 v^3 + 5 o^3 v^2) flops
(7.71e13 at 60/240), whatever the kernels actually execute.

Also reported (measured once per run, outside the timed steps): the full
mixed-precision solve (3xTF32 iterations, one FP64-accurate base residual with
Ozaki-split bf16 tensor-core GEMMs, defect correction) to the reference's
convergence test; the plain FP64 GPU solve of the same problem to the same test
(wall time, |dE| and the largest amplitude difference between the two); the
FP64 residual norm at the mixed solution (a-posteriori check); the same
comparison at o/v = 40/160; and the reference path's CPU rate (the NumPy oracle
on the host cores) on a bounded sample of this workload (``cpu_residual_sample``).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
       python bench.py --profile gemm|jk|hbm ...   (one kernel on a small case)
Multi-GPU: replicas only (each rank solves its own copy; no collective on the
data path); value = sum of per-rank work / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def alg_flops(o, v):
    return 8.0 * (0.5 * o * o * v ** 4 + o ** 3 * v ** 3 + 0.5 * o ** 4 * v * v + 5 * o * o * v ** 3 + 5 * o ** 3 * v * v)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_info():
    ncores = len(os.sched_getaffinity(0))
    try:
        ram = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES") / 1e9
    except (ValueError, OSError):
        ram = None
    return ncores, ram


# Virtual rows per CPU sample step: about 1/120 (60/240) and 1/40 (40/160) of a residual.
SAMPLE_ROWS = {(60, 240): 2, (40, 160): 4}


def cpu_residual_sample(o, v, steps, warmup=1, rows=None, seed=0):
    """The reference path's residual (the NumPy oracle's restatement of
    apyib/ci_wfn.py:309-334, opt_einsum-style full-tensor contractions) timed on the
    host cores at o/v on a bounded sample: each step evaluates the residual rows of
    ``rows`` virtual indices a (r1[:, a], r2[:, :, a, :]), every einsum of the
    reference restricted to those output rows with its full contraction lengths, so
    a step does rows / v of the residual's work on the workload's own shapes.  The
    integral blocks are the seeded synthetic problem's (vvvv, vovv, vvvo, vvoo for the
    sampled rows; ovvo, ooov, ovoo, oooo in full) and the amplitudes those of the first
    iteration (t1 = 0, t2 = <ab||ij> / D), all built before the timed steps, as are the
    full-size operands' relayouts (``oracle.port.vslab_layouts``): the reference's
    einsums copy them once per term and residual, which the sample cannot scale, so the
    implied full-residual time leaves those copies out and favours the CPU.
    Returns per-step seconds and a description."""
    import importlib
    ncores, ram = host_info()
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ.setdefault(k, str(ncores))
    port = importlib.import_module("oracle.port")
    from apyib_gb300 import synthetic
    rows = rows or SAMPLE_ROWS.get((o, v), max(1, v // 120))
    prob = synthetic.so_factors(o, v, seed=seed)
    F = prob.fock_so()
    t_set = time.perf_counter()
    blk = port.vslab_blocks_from_factors(prob.B, o, 0, rows)
    # amplitudes of the first iteration: t1 = 0, t2 = <ab||ij> / D (full o, o, v, v)
    D_ia, D_ijab = port.so_denominators(prob.eps_o, prob.eps_v)
    step_v = 16
    vvoo = np.concatenate([port.vslab_blocks_from_factors(prob.B, o, b0, min(v, b0 + step_v), names=("vvoo",))["vvoo"]
                           for b0 in range(0, v, step_v)])
    t2 = vvoo.transpose(2, 3, 0, 1) / D_ijab
    t1 = np.zeros((o, v), dtype=complex)
    del vvoo, D_ijab, prob
    lay = port.vslab_layouts(blk, t2)
    setup_s = time.perf_counter() - t_set
    times = []
    for step in range(warmup + steps):
        c0 = time.perf_counter()
        port.cisd_so_residual_vslab(F, blk, t1, t2, 0.1, o, 0, rows, lay=lay)
        dt = time.perf_counter() - c0
        if step >= warmup:
            times.append(dt)
    frac = rows / v
    return {"step_s": times, "rows": rows, "fraction": frac, "cores": ncores, "host_ram_GB": ram,
            "setup_s": setup_s,
            "sample": f"residual rows of {rows} of {v} virtual indices per step (every reference einsum of "
                      f"apyib/ci_wfn.py:309-334 restricted to them, full contraction lengths, operand relayouts "
                      f"done once before timing; {frac:.4f} of the residual's work) at o/v={o}/{v}, NumPy oracle "
                      f"port, {ncores} host cores; value = algorithmic flops / (step time / {frac:.4f})"}


def cpu_baseline_oracle(o=60, v=240, steps=3):
    """CPU baseline of the bench line: ``cpu_residual_sample`` at the bench's o/v."""
    r = cpu_residual_sample(o, v, steps)
    dt = float(np.mean(r["step_s"]))
    full_s = dt / r["fraction"]
    return {"value": alg_flops(o, v) / full_s / 1e12, "unit": "TFLOP/s", "cores": r["cores"], "kind": "port",
            "sample": r["sample"] + f"; {dt:.2f} s per step",
            "full_residual_s_from_sample": full_s, "host_ram_GB": r["host_ram_GB"], "setup_s": r["setup_s"]}


def bench_config(o, v, world):
    return {"workload": f"CISD_SO mixed-precision iteration, synthetic o/v={o}/{v} spin orbitals",
            "o": o, "v": v, "naux": 4 * (o + v), "l2": "inputs > L2 (ERI blocks ~45 GB in HBM)",
            "parallelism": f"replicas x{world}", "alg_flops_per_step": alg_flops(o, v)}


def run_reference(args, rank, world):
    """The reference arm: the reference path on the host cores (the NumPy oracle's
    restatement, as the reference itself is Python that imports psi4 at module
    level), on this bench's workload and metric; each step is one bounded sample
    (``cpu_residual_sample``) and its value the residual's algorithmic flops over the
    time of a full residual implied by the sample.  Rank 0 only."""
    if rank != 0:
        return 0
    o, v = args.o, args.v
    r = cpu_residual_sample(o, v, args.steps, warmup=args.warmup)
    step_s = float(np.mean(r["step_s"]))
    full_s = step_s / r["fraction"]
    val = alg_flops(o, v) / full_s / 1e12
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": bench_config(o, v, world),
            "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": r["cores"], "kind": "port",
                             "sample": r["sample"], "full_residual_s_from_sample": full_s,
                             "host_ram_GB": r["host_ram_GB"], "setup_s": r["setup_s"]},
            "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def ao_kernels(nbf, seed=0):
    """J/K Fock build and AO->MO transform at nbf basis functions (real AO ERIs from
    random real symmetric factors, complex unitary C), timed with CUDA events."""
    import ctypes

    import torch

    from apyib_gb300 import _lib
    from apyib_gb300.device import ptr, stream_ptr, workspace
    g = torch.Generator(device="cpu").manual_seed(seed)
    naux = 3 * nbf
    A = torch.randn(naux, nbf, nbf, generator=g, dtype=torch.float64)
    A = (A + A.transpose(1, 2)) / (2 * (naux * nbf) ** 0.5)
    eri = torch.einsum("Lmn,Lls->mnls", A.cuda(), A.cuda())
    eri = (0.5 * (eri + eri.transpose(2, 3))).contiguous()      # exactly symmetric in (l, s), as AO ERIs are
    X = torch.randn(nbf, nbf, generator=g, dtype=torch.complex128)
    C = torch.linalg.qr(X)[0].cuda().contiguous()
    D = (C[:, : nbf // 4] @ C[:, : nbf // 4].conj().T).contiguous()
    h = torch.zeros(nbf, nbf, dtype=torch.complex128, device="cuda")
    F = torch.empty_like(h)
    res = {}

    def timed(fn, n=3):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n / 1e3

    njk = _lib.load().agb_jk_fock_scratch_bytes(nbf)
    jbuf, jsp, _ = workspace(njk)
    t = timed(lambda: _lib.call("agb_jk_fock", ptr(eri), nbf, ptr(D), ptr(h), 1.0, ptr(F), ctypes.c_void_p(jsp),
                                ctypes.c_size_t(njk), stream_ptr()))
    peaks, _ = measured_peaks()
    gbs = 8.0 * nbf ** 4 / t / 1e9
    res["jk_fock"] = {"ms": t * 1e3, "eri_GB": 8.0 * nbf ** 4 / 1e9, "achieved_GBps": gbs,
                      "hbm_peak_GBps": peaks["hbm_gbs"], "frac": gbs / peaks["hbm_gbs"]}
    F_gen = F.clone()
    t = timed(lambda: _lib.call("agb_jk_fock_sym", ptr(eri), nbf, ptr(D), ptr(h), 1.0, ptr(F), ctypes.c_void_p(jsp),
                                ctypes.c_size_t(njk), stream_ptr()))
    gbs = 8.0 * nbf ** 4 / t / 1e9
    res["jk_fock_sym"] = {"ms": t * 1e3, "eri_GB_read": 4.0 * nbf ** 3 * (nbf + 1) / 1e9, "achieved_GBps": gbs,
                          "frac": gbs / peaks["hbm_gbs"],
                          "max_abs_diff_vs_general": (F - F_gen).abs().max().item(),
                          "note": "ERIs symmetric in (l, s): the l <= s half is read; achieved counts the "
                                  "full tensor the result depends on (8 nbf^4 B)"}
    F_df = F.clone()
    t = timed(lambda: _lib.call("agb_jk_fock_sym64", ptr(eri), nbf, ptr(D), ptr(h), 1.0, ptr(F),
                                ctypes.c_void_p(jsp), ctypes.c_size_t(njk), stream_ptr()))
    res["jk_fock_sym64"] = {"ms": t * 1e3, "arith": "fp64 (6 DFMA per pair of integrals)",
                            "max_abs_diff_vs_df": (F - F_df).abs().max().item()}
    out = torch.empty(nbf, nbf, nbf, nbf, dtype=torch.complex128, device="cuda")
    flops = 2.0 * 2 * nbf ** 5 + 3 * 8.0 * nbf ** 5    # real x complex first step, then three complex steps
    ref = None
    for name, prec in (("fp64", _lib.PREC_FP64), ("df64", _lib.PREC_DF64), ("ozaki", _lib.PREC_OZAKI),
                       ("tf32x3", _lib.PREC_TF32X3)):
        nb = _lib.load().agb_ao2mo_scratch_bytes(nbf, nbf, prec)
        buf, sp, _ = workspace(nb)
        t = timed(lambda: _lib.call("agb_ao2mo", ptr(eri), nbf, ptr(C), nbf, ptr(out), ctypes.c_void_p(sp),
                                    ctypes.c_size_t(nb), prec, stream_ptr()), n=1)
        res[f"ao2mo_{name}"] = {"ms": t * 1e3, "TFLOPs": flops / t / 1e12}
        if ref is None:
            ref = out[:20].clone()
        else:
            res[f"ao2mo_{name}"]["max_abs_diff_vs_fp64"] = (out[:20] - ref).abs().max().item()
        del buf
    del out, eri, jbuf, ref
    torch.cuda.empty_cache()
    return res


H2O_GEOM = """
O 0.0  0.0     0.1173
H 0.0  0.7572 -0.4692
H 0.0 -0.7572 -0.4692
units angstrom
no_com
no_reorient
symmetry c1
"""


def water_workloads():
    """Water cc-pVDZ with a 1e-4 a.u. magnetic field along z (complex orbitals), from
    the geometry string through the public API: the CISD_SO solve in FP64 and in
    mixed precision, and the finite-difference AAT tensor (9 nuclear coordinates x
    3 field components, steps 1e-4 bohr and 1e-5 a.u.: 24 displaced CISD solves,
    the MO overlaps and the determinant-overlap terms as contractions).  Beside it,
    the reference's determinant path for the same tensor: the number of o x o
    determinants its loops evaluate (apyib/aats.py:161-555) times the rate of
    batched 10 x 10 complex determinants measured here on the host (an estimate:
    the path itself would run for months).  At zero field: the analytic nuclear
    gradient and the atomic polar tensor from six analytic gradients, each against
    its finite-difference counterpart on the same GPU path."""
    import torch

    from apyib_gb300.aats import AAT
    from apyib_gb300.energy import energy
    from apyib_gb300.fin_diff import finite_difference
    from apyib_gb300.hamiltonian import Hamiltonian
    from apyib_gb300.hf_wfn import hf_wfn

    p = dict(geom=H2O_GEOM, basis="cc-pVDZ", method="CISD_SO", e_convergence=1e-10, d_convergence=1e-10,
             DIIS=True, max_iterations=120, freeze_core=False, F_el=[0.0, 0.0, 0.0], F_mag=[0.0, 0.0, 1e-4])
    from apyib_gb300.ci_wfn import ci_wfn
    energy(dict(p, method="RHF"))                      # warm-up: library load, first kernels
    res, phases = {}, {}
    for prec in ("fp64", "mixed"):
        pp = dict(p, precision=prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E_list, T_list, C, basis = energy(pp)
        torch.cuda.synchronize()
        res[prec] = (time.perf_counter() - t0, complex(E_list[1]))
        # the same run phase by phase: AO integrals, RHF, F_MO + AO->MO transform, CISD_SO solve
        marks = [time.perf_counter()]
        H = Hamiltonian(pp)
        torch.cuda.synchronize()
        marks.append(time.perf_counter())
        wfn = hf_wfn(H)
        wfn.solve_SCF(pp)
        torch.cuda.synchronize()
        marks.append(time.perf_counter())
        ci = ci_wfn(pp, wfn)
        torch.cuda.synchronize()
        marks.append(time.perf_counter())
        ci.solve_CISD_SO()
        torch.cuda.synchronize()
        marks.append(time.perf_counter())
        phases[prec] = {name: marks[i + 1] - marks[i]
                        for i, name in enumerate(("integrals_s", "rhf_s", "fock_and_transform_s", "cisd_so_solve_s"))}
    out = {"cisd_fp64_s": res["fp64"][0], "cisd_mixed_s": res["mixed"][0],
           "E_cisd": [res["fp64"][1].real, res["fp64"][1].imag],
           "abs_dE_mixed_vs_fp64": abs(res["mixed"][1] - res["fp64"][1]),
           "phases": phases,
           "note": "nso = 48: launch-bound at this size; the solves include integrals and RHF; phases: the "
                   "same run split into AO integrals, RHF, F_MO + AO->MO transform (FP64 / Ozaki) and the "
                   "CISD_SO solve (FP64 / mixed)"}
    h, b = 1e-4, 1e-5
    E_list, T_list, C, basis = energy(p)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fd = finite_difference(p, basis, C)
    inputs = fd.compute_AAT(h, b)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    A = AAT(p, hf_wfn(Hamiltonian(p)), C, basis, T_list, *inputs, h, b)
    aat = A.compute_aat_tensor("full")
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    o, v = 10, 38
    ov = o * v
    dets_per_element = 4 + 2 * 6 * ov * ov + 9 * ov ** 4 + 2 * 9 * ov ** 3 + 9 * ov * ov + 2 * 6 * ov
    rng = np.random.default_rng(0)
    M = rng.standard_normal((20000, o, o)) + 1j * rng.standard_normal((20000, o, o))
    np.linalg.det(M[:100])
    c0 = time.perf_counter()
    np.linalg.det(M)
    rate = len(M) / (time.perf_counter() - c0)
    out["aat_fd"] = {"total_s": t2 - t0, "displaced_solves": len(inputs[0]) * 2 + 6, "solves_s": t1 - t0,
                     "overlaps_and_terms_s": t2 - t1, "elements": int(aat.size), "max_abs_element": float(
                         np.abs(aat).max()),
                     "reference_determinants": 27 * dets_per_element,
                     "reference_estimate_s": 27 * dets_per_element / rate,
                     "cpu_det_rate_per_s": rate, "cpu_cores": 1,
                     "cpu_sample": "20000 batched 10x10 complex determinants (numpy), one host thread"}
    # nuclear derivatives at zero field: analytic (one SCF + one CI solve, densities, derivative
    # integrals, CPHF) against central differences of complete solves
    from apyib_gb300.gradient import apt, nuclear_gradient
    p0 = dict(p, F_mag=[0.0, 0.0, 0.0])
    nuclear_gradient(dict(p0, basis="STO-3G"))                   # warm-up of the derivative kernels
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g_an = nuclear_gradient(p0)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    E_list, T_list, C, basis = energy(p0)
    fd0 = finite_difference(p0, basis, C)
    t2 = time.perf_counter()
    g_fd = fd0.compute_Nuclear_Gradient(1e-4)[0]
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    P_an = apt(p0)
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    P_fd = fd0.compute_APT(1e-3, 1e-4)
    torch.cuda.synchronize()
    t5 = time.perf_counter()
    from apyib_gb300.analytic_aats import analytic_derivative
    analytic_derivative(dict(p0, basis="STO-3G")).compute_CISD_AATs()      # warm-up
    analytic_derivative(dict(p0, basis="STO-3G")).compute_CISD_AATs(precision="mixed")
    torch.cuda.synchronize()
    t6 = time.perf_counter()
    aat_an = analytic_derivative(p0).compute_CISD_AATs(normalization="full")
    torch.cuda.synchronize()
    t7 = time.perf_counter()
    aat_mx = analytic_derivative(p0).compute_CISD_AATs(normalization="full", precision="mixed")
    torch.cuda.synchronize()
    t7m = time.perf_counter()
    inputs0 = fd0.compute_AAT(1e-4, 1e-4)
    aat_fd = AAT(p0, hf_wfn(Hamiltonian(p0)), C, basis, T_list, *inputs0, 1e-4, 1e-4).compute_aat_tensor("full")
    torch.cuda.synchronize()
    t8 = time.perf_counter()
    out["derivatives_zero_field"] = {
        "gradient_analytic_s": t1 - t0, "gradient_fd_s": t3 - t2, "gradient_fd_solves": 18,
        "gradient_max_abs_diff": float(np.abs(g_an - g_fd).max()),
        "apt_semianalytic_s": t4 - t3, "apt_analytic_gradients": 12, "apt_fd_s": t5 - t4, "apt_fd_energies": 108,
        "apt_max_abs_diff": float(np.abs(P_an - P_fd.real).max()),
        "aat_analytic_s": t7 - t6, "aat_analytic_mixed_s": t7m - t7,
        "aat_analytic_mixed_max_abs_diff": float(np.abs(aat_mx - aat_an).max()),
        "aat_analytic_responses": 12, "aat_fd_s": t8 - t7m, "aat_fd_solves": 24,
        "aat_max_abs_diff": float(np.abs(aat_an - aat_fd).max()),
        "note": "water cc-pVDZ CISD_SO, zero field; FD steps 1e-4 bohr (gradient, AAT), 1e-3 bohr / 1e-4 a.u. "
                "(APT), 1e-4 a.u. (AAT); semianalytic APT = analytic gradients at +-h, +-2h of each field "
                "component (Richardson, h = 5e-4 a.u.); analytic AAT = one solve, nuclear + magnetic CPHF, 3N+3 "
                "amplitude responses"}
    return out


def hbm_kernels(plan, t, diis, hbm_gbs, reps=5):
    """The HBM-bound kernels of an iteration at the bench's o/v, each timed alone with
    CUDA events (mean of `reps` launches after one warm-up) against its algorithmic
    bytes (complex128 = 16 B per element of the packed amplitude vector, n1 + n2
    elements): the amplitude update (apyib/ci_wfn.py:336-337) reads t, r and writes
    t_new (48 B); the DIIS Gram row with the full history (apyib/utils.py:121) reads
    x and the 8 stored vectors (144 B); the DIIS combination fused with the energy and
    step norms (apyib/utils.py:138 + ci_wfn.py:355,361-365) reads 8 vectors, t_old and
    the energy weights and writes t_new (176 B); MP2_SO (apyib/mp2_wfn.py:82-85) reads
    the packed <ab||ij> and energy weights and writes t2 (48 B per packed doubles
    element)."""
    import torch
    n, n2 = plan.n1 + plan.n2, plan.n2
    r = t.clone()                                  # any vector of the right length
    ys = list(diis.t)[:8]
    ys += [t] * (8 - len(ys))
    out3 = torch.empty(16, dtype=torch.complex128, device=t.device)
    tn = torch.empty_like(t)
    c = [1.0 / len(ys)] * len(ys)
    cases = {
        "update": (lambda: plan.update(t, r, out=tn), 48 * n),
        "diis_gram_row_8": (lambda: plan.dots_into(t, ys, out3), 16 * 9 * n),
        "diis_combine_8": (lambda: plan.combine_into(ys, c, t, tn, out3), 16 * 11 * n),
        "mp2_so": (lambda: plan.mp2_into(tn, out3), 48 * n2),
    }
    res = {}
    for name, (fn, nbytes) in cases.items():
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        gbs = nbytes / ms / 1e6
        res[name] = {"ms": ms, "alg_GB": nbytes / 1e9, "achieved_GBps": gbs, "frac": gbs / hbm_gbs}
    res["peak_GBps"] = hbm_gbs
    res["note"] = "CUDA events around each call alone (its reduction tail included), mean of 5, inputs > L2"
    del r, tn
    return res


def mixed_iteration(plan):
    """One mixed-precision CISD_SO iteration as the bench times it: 3xTF32 residual,
    FP64 update, DIIS push (Gram row) and the FP64 extrapolation with energy and norms."""
    from apyib_gb300 import _lib
    from apyib_gb300.cisd import _DIIS
    t = plan.guess()
    E, _, _ = plan.combine([t], [1.0], t, t)
    diis = _DIIS(plan)
    state = {"t": t, "E": E, "first": True}

    def iteration():
        r = plan.residual(state["t"], state["E"], _lib.PREC_TF32X3)
        tn = plan.update(state["t"], r)
        diis.push(r, tn, state["first"])
        state["first"] = False
        c = diis.coefficients()
        E, s1, s2 = plan.combine(diis.t, c, state["t"], state["t"])
        state["E"] = E
        return E
    return iteration, state, diis


def gemm_traffic_60_240():
    """DRAM bytes per launch of the bench's two tensor-core GEMMs at o/v = 60/240 (the ring
    GEMM 14400 x 14400 x 14400 and the vvvv ladder 1770 x 28680 x 28680, complex), mean of
    the two.  Counters are taken on smaller GEMMs with the same K and the same 256 x 256
    pair tiles, which hold a few GB on the device (profiles/tf32x3_gemm_traffic_small.md):
    3584 x 3584 x 14400 read 3.893e9 B over 14 x 14 pair tiles, 1770 x 3584 x 28680 read
    3.411e9 B over 7 x 14.  Each tile streams its own A and B panels through L2, so the
    read traffic is scaled by the pair-tile count of the full launch (57 x 57 and 7 x 113);
    the output is counted as written once (16 B per element)."""
    ring = 3.893e9 / (14 * 14) * (57 * 57) + 16.0 * 14400 * 14400
    vvvv = 3.411e9 / (7 * 14) * (7 * 113) + 16.0 * 1770 * 28680
    return 0.5 * (ring + vvvv)


def timed_iterations(iteration, steps, warmup):
    import torch
    for _ in range(warmup):
        iteration()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        iteration()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def gpu_numa_cpus(dev_index):
    """(NUMA node of the GPU's PCI function, the usable host cores on that node) from sysfs;
    (None, []) when the system does not say."""
    import torch
    try:
        bdf = torch.cuda.get_device_properties(dev_index).pci_bus_id.lower()
    except Exception:
        bdf = None
    if not bdf:
        try:
            out = subprocess.run(["nvidia-smi", "-i", str(dev_index), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                                 capture_output=True, text=True, timeout=20).stdout.strip().lower()
            bdf = out[4:] if len(out) > 12 else out       # 00000000:xx:yy.z -> 0000:xx:yy.z
        except Exception:
            return None, []
    try:
        with open(f"/sys/bus/pci/devices/{bdf}/numa_node") as f:
            node = int(f.read().strip())
        if node < 0:
            return None, []
        with open(f"/sys/devices/system/node/node{node}/cpulist") as f:
            cpus = set()
            for part in f.read().strip().split(","):
                a, _, b = part.partition("-")
                cpus.update(range(int(a), int(b or a) + 1))
    except (OSError, ValueError):
        return None, []
    return node, sorted(cpus & os.sched_getaffinity(0))


def pinned_local(n, dtype, dev_index):
    """Pinned host buffers placed on the GPU's NUMA node: allocated and first touched by
    this thread while it runs on that node's cores (the kernel places pages where they
    are first touched), so host<->GPU copies do not cross the socket link.  Returns the
    tensors and the node (None when the node or its cores are not available)."""
    import torch
    node, cpus = gpu_numa_cpus(dev_index)
    old = os.sched_getaffinity(0)
    try:
        if cpus:
            os.sched_setaffinity(0, cpus)
        bufs = [torch.empty(n, dtype=dtype, pin_memory=True) for _ in range(2)]
        for b in bufs:
            b.zero_()
    finally:
        if cpus:
            os.sched_setaffinity(0, old)
    return bufs, (node if cpus else None)


def max_over_ranks(x, dist=None):
    """Max of a per-rank scalar over all ranks (identity without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_throughput(world, work_per_rank, max_seconds):
    """Whole-job throughput of independent replicas: total work / slowest rank."""
    return world * work_per_rank / max_seconds


def profile_kernel(spec):
    """One kernel on a small case, for timing and for an ncu capture (``--profile``):

        gemm M N K [tf32x3|df64|oz|fp64]   complex GEMM, A [M,K], B used transposed [N,K]
        jk NBF REPS [sym|sym64|general]    J/K Fock build over seeded real AO integrals
        ao2mo NBF [ozaki|tf32x3|df64|fp64] the AO->MO transform, nmo = nbf
        hbm O V [update|dots|combine|mp2]  the amplitude update, DIIS Gram row (8 vectors),
                                           DIIS combination (8 vectors) and MP2_SO at o/v
                                           spin orbitals (each once timed, after two runs)

    Each case runs twice untimed, then once (gemm) or REPS / 3 times under CUDA events,
    and prints one line."""
    import ctypes

    import torch

    from apyib_gb300 import _lib
    from apyib_gb300.device import ptr, stream_ptr, workspace
    torch.cuda.set_device(0)
    kind, args = spec[0], spec[1:]
    if kind == "gemm":
        M, N, K = (int(a) for a in args[:3])
        prec = args[3] if len(args) > 3 else "tf32x3"
        g = torch.Generator(device="cuda").manual_seed(0)
        A = torch.randn(M, K, dtype=torch.complex128, device="cuda", generator=g)
        B = torch.randn(N, K, dtype=torch.complex128, device="cuda", generator=g)
        C = torch.zeros(M, N, dtype=torch.complex128, device="cuda")
        size_fn = {"tf32x3": "agb_cgemm_tf32x3_scratch_bytes", "df64": "agb_zgemm_df64_scratch_bytes",
                   "oz": "agb_zgemm_oz_scratch_bytes"}.get(prec)
        nb = getattr(_lib.load(), size_fn)(M, N, K) if size_fn else 256
        buf, sp, _ = workspace(nb)
        buf.zero_()
        entry = {"tf32x3": "agb_cgemm_tf32x3", "df64": "agb_zgemm_df64_ex", "oz": "agb_zgemm_oz"}.get(prec)

        def run():
            if entry:
                _lib.call(entry, M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                          ctypes.c_void_p(sp), ctypes.c_size_t(nb), stream_ptr())
            else:
                _lib.call("agb_zgemm", M, N, K, 1.0, 0.0, ptr(A), K, 1, 0, ptr(B), 1, K, 0, 0.0, 0.0, ptr(C), N,
                          stream_ptr())
        reps, work, label = 1, 8.0 * M * N * K, f"gemm {prec} {M}x{N}x{K}"
    elif kind == "jk":
        from apyib_gb300.linalg import jk_fock
        n = int(args[0]) if args else 150
        reps = int(args[1]) if len(args) > 1 else 5
        variant = args[2] if len(args) > 2 else "sym"
        g = torch.Generator(device="cpu").manual_seed(0)
        A = torch.randn(3 * n, n, n, generator=g, dtype=torch.float64)
        A = ((A + A.transpose(1, 2)) / (2 * (3 * n * n) ** 0.5)).cuda()
        eri = torch.einsum("Lmn,Lls->mnls", A, A)
        del A
        eri = (0.5 * (eri + eri.transpose(2, 3))).contiguous()
        if variant == "general":
            eri[0, 0, 0, 1] = eri[0, 0, 0, 1] * (1 + 2.0 ** -40) + 1e-300   # not (l, s)-symmetric
        Cm = torch.linalg.qr(torch.randn(n, n, generator=g, dtype=torch.complex128))[0].cuda()
        D = (Cm[:, : n // 4] @ Cm[:, : n // 4].conj().T).contiguous()
        h = torch.zeros(n, n, dtype=torch.complex128, device="cuda")
        prec = "fp64" if variant == "sym64" else "df64"

        def run():
            jk_fock(eri, D, h, 1.0, precision=prec)
        work, label = 8.0 * n ** 4, f"jk_fock {variant} nbf={n} (GB/s of the full ERI tensor)"
    elif kind == "ao2mo":
        n = int(args[0]) if args else 96
        prec_name = args[1] if len(args) > 1 else "ozaki"
        prec = {"fp64": _lib.PREC_FP64, "df64": _lib.PREC_DF64, "ozaki": _lib.PREC_OZAKI,
                "tf32x3": _lib.PREC_TF32X3}[prec_name]
        g = torch.Generator(device="cpu").manual_seed(0)
        A = torch.randn(3 * n, n, n, generator=g, dtype=torch.float64)
        A = ((A + A.transpose(1, 2)) / (2 * (3 * n * n) ** 0.5)).cuda()
        eri = torch.einsum("Lmn,Lls->mnls", A, A).contiguous()
        del A
        Cm = torch.linalg.qr(torch.randn(n, n, generator=g, dtype=torch.complex128))[0].cuda().contiguous()
        out = torch.empty(n, n, n, n, dtype=torch.complex128, device="cuda")
        nb = _lib.load().agb_ao2mo_scratch_bytes(n, n, prec)
        buf, sp, _ = workspace(nb)

        def run():
            _lib.call("agb_ao2mo", ptr(eri), n, ptr(Cm), n, ptr(out), ctypes.c_void_p(sp), ctypes.c_size_t(nb), prec,
                      stream_ptr())
        reps, work, label = 1, 28.0 * n ** 5, f"ao2mo {prec_name} nbf={n} (TFLOP/s of 28 nbf^5)"
    elif kind == "hbm":
        from apyib_gb300 import synthetic
        from apyib_gb300.cisd import CISDPlan
        o, v = int(args[0]), int(args[1])
        which = args[2] if len(args) > 2 else "all"
        prob = synthetic.so_factors(o, v, seed=0)
        eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
        # these kernels read only the vectors, 1/D and the energy weights: an MP2 plan
        # (two packed integral blocks) keeps the device footprint small
        plan = CISDPlan(o, v, mp2_only=True)
        plan.set_fock(torch.as_tensor(prob.fock_so()), eps_so)
        plan.blocks_from_factors(torch.as_tensor(prob.B), precision=_lib.PREC_DF64)
        t = torch.zeros(plan.n, dtype=torch.complex128, device="cuda")
        plan.mp2_into(t, torch.empty(16, dtype=torch.complex128, device="cuda"))
        g = torch.Generator(device="cuda").manual_seed(1)
        ys = [t + 1e-3 * torch.randn(t.shape, dtype=t.dtype, device=t.device, generator=g) for _ in range(8)]
        out3 = torch.empty(16, dtype=torch.complex128, device=t.device)
        tn = torch.empty_like(t)
        n, n2 = plan.n1 + plan.n2, plan.n2
        cases = {"update": (lambda: plan.update(t, ys[0], out=tn), 48 * n),
                 "dots": (lambda: plan.dots_into(t, ys, out3), 16 * 9 * n),
                 "combine": (lambda: plan.combine_into(ys, [0.125] * 8, t, tn, out3), 16 * 11 * n),
                 "mp2": (lambda: plan.mp2_into(tn, out3), 48 * n2)}
        sel = cases if which == "all" else {which: cases[which]}
        for name, (fn, nbytes) in sel.items():
            fn()
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            print(f"ok hbm {name} o/v={o}/{v}: {ms:.3f} ms, {nbytes / ms / 1e6:.0f} GB/s of {nbytes / 1e9:.3f} GB")
        plan.check_status()
        return 0
    else:
        raise SystemExit(f"unknown --profile kind {kind!r}")
    run()
    run()
    if kind == "gemm" and prec in ("tf32x3", "oz"):
        _lib.call("agb_scratch_status", ctypes.c_void_p(sp), stream_ptr())
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    unit = {"gemm": "TFLOP/s (8MNK)", "ao2mo": "TFLOP/s"}.get(kind, "GB/s")
    scale = 1e9 if kind in ("gemm", "ao2mo") else 1e6
    print(f"ok {label}: {ms:.3f} ms, {work / ms / scale:.1f} {unit}")
    return 0


METRIC = "CISD_SO iteration TFLOP/s (algorithmic), mixed 3xTF32 + FP64 refinement, synthetic o/v=60/240"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--o", type=int, default=60)
    ap.add_argument("--v", type=int, default=240)
    ap.add_argument("--no-solve", action="store_true", help="skip the once-per-run full solve")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-fp64-solve", action="store_true",
                    help="skip the full FP64 GPU solve at the bench shape (several minutes at 60/240)")
    ap.add_argument("--profile", nargs="+", metavar="ARG",
                    help="run one kernel on a small case instead of the bench (see profile_kernel)")
    args = ap.parse_args()
    if args.profile:
        return profile_kernel(args.profile)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import ctypes

    import torch

    from apyib_gb300 import _lib, synthetic
    from apyib_gb300.cisd import CISDPlan, _DIIS, solve
    from apyib_gb300.device import ptr, stream_ptr

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = _lib.load()
    o, v = args.o, args.v
    W = alg_flops(o, v)
    prob = synthetic.so_factors(o, v, seed=0)
    eps_so = np.concatenate([np.repeat(prob.eps_o, 2), np.repeat(prob.eps_v, 2)])
    t_setup = time.perf_counter()
    plan = CISDPlan(o, v, mixed=True)
    plan.set_fock(torch.as_tensor(prob.fock_so()), eps_so)
    # integral blocks from the factors: the large products on the bf16 tensor cores with
    # six-slice Ozaki splitting (~1e-12 of sum |a||b|), the rest in double-float; every
    # solve below uses these same blocks
    plan.blocks_from_factors(torch.as_tensor(prob.B), precision=_lib.PREC_OZAKI)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    del prob

    # ---- iteration state
    iteration, state, diis = mixed_iteration(plan)

    for _ in range(args.warmup):
        iteration()
    plan.check_status()
    torch.cuda.synchronize()

    # ---- timed device-resident steps
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    _lib.call("agb_cisd_plan_gemm_timing", plan._h, 1)
    n0 = lib.agb_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        iteration()
    ev1.record()
    torch.cuda.synchronize()
    launches = lib.agb_launch_count() - n0
    _lib.call("agb_cisd_plan_gemm_timing", plan._h, 0)
    nl, kms, kfl = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
    pq = (o * (o - 1) // 2) * (v * (v - 1) // 2) ** 2       # vvvv ladder M*N*K
    ring = float(o * v) ** 3
    _lib.call("agb_cisd_plan_gemm_timing_collect", plan._h, min(pq, ring) * 0.99, ctypes.byref(nl), ctypes.byref(kms),
              ctypes.byref(kfl))
    plan.check_status()
    dev_ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, dist)
    clocks = sampler.stop()

    # ---- e2e: iterations whose amplitude vectors live in pinned host memory.  Two
    # independent iterates (the bench's and a second one started from the same guess)
    # alternate on the compute stream; every step copies its iterate in (H2D) before
    # the iteration and its result out (D2H) after it, on a copy stream, so one
    # iterate's copies overlap the other's iteration.  The device buffers of the two
    # iterates are the ping-pong pair; the pinned buffers sit on the GPU's NUMA node.
    it_b, state_b, diis_b = mixed_iteration(plan)
    for _ in range(args.warmup):
        it_b()
    chains = [(iteration, state), (it_b, state_b)]
    bufs = []
    for c in range(2):
        pair, numa_node = pinned_local(plan.n, torch.complex128, local)
        pair[0].copy_(chains[c][1]["t"].cpu())            # the iterate starts on the host
        bufs.append(pair)                                 # [input, output] of chain c
    copy = torch.cuda.Stream()
    # the vector crosses in 32 pieces, so a small blocking read-back of the iteration (its
    # DIIS Gram row and energy) queues behind one piece, not behind the whole vector, on
    # the shared device-to-host copy engine
    pieces = [(a, min(plan.n, a + (plan.n + 31) // 32)) for a in range(0, plan.n, (plan.n + 31) // 32)]

    def copy_pieces(dst, src):
        for a, b in pieces:
            dst[a:b].copy_(src[a:b], non_blocking=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    comp = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(comp)
    copy.wait_event(e0)
    ready, h2d_ev, d2h_ev = [None, None], [], []
    for c in range(min(2, args.steps)):
        with torch.cuda.stream(copy):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(copy)
            copy_pieces(chains[c][1]["t"], bufs[c][0])
            b.record(copy)
            h2d_ev.append((a, b))
            ready[c] = b
    for k in range(args.steps):
        c = k % 2
        comp.wait_event(ready[c])
        chains[c][0]()
        done = torch.cuda.Event()
        done.record(comp)
        with torch.cuda.stream(copy):
            copy.wait_event(done)
            a, b, d = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            a.record(copy)
            copy_pieces(bufs[c][1], chains[c][1]["t"])                   # D2H: the step's result
            b.record(copy)
            bufs[c][0], bufs[c][1] = bufs[c][1], bufs[c][0]               # the result is the next input
            d2h_ev.append((a, b))
            if k + 2 < args.steps:                                       # this iterate runs again at step k + 2
                copy_pieces(chains[c][1]["t"], bufs[c][0])               # H2D: that step's input
                d.record(copy)
                h2d_ev.append((b, d))
                ready[c] = d
    comp.wait_stream(copy)
    e1.record(comp)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dist)
    h2d_ms = float(np.mean([a.elapsed_time(b) for a, b in h2d_ev]))
    d2h_ms = float(np.mean([a.elapsed_time(b) for a, b in d2h_ev]))
    nbytes = plan.n * 16
    del it_b, state_b, diis_b, chains, bufs

    peaks, peak_kind = measured_peaks()
    tf32_peak = peaks["bf16_tflops"] / 2.0        # tcgen05 kind::tf32 issues at half the f16/bf16 rate
    gemm_peak = tf32_peak / 3.0                   # 3 TF32 products per FP32 product
    kern_ach = (kfl.value / (kms.value / 1e3) / 1e12) if kms.value > 0 else None

    out = {
        "metric": METRIC, "value": aggregate_throughput(world, W, dev_ms / 1e3) / 1e12, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 (3xTF32 tensor core) + c128 (update/DIIS/sums)",
        "data": f"synthetic (seeded Hermitian factors, o/v={o}/{v}; the headline shape is 60/240)",
        "config": bench_config(o, v, world),
        "e2e": {"value": aggregate_throughput(world, W, e2e_ms / 1e3) / 1e12, "unit": "TFLOP/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                # copies on the copy stream, overlapping the other iterate's iteration
                "h2d_ms": h2d_ms, "d2h_ms": d2h_ms,
                "h2d_GBps": nbytes / h2d_ms / 1e6, "d2h_GBps": nbytes / d2h_ms / 1e6,
                "pinned_numa_node": numa_node,
                "pipeline": "two independent iterates alternate on the compute stream; each step copies its "
                            "iterate in from pinned host memory before the iteration and its result out after "
                            "it, on a copy stream that overlaps the other iterate's iteration"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "tensor", "kernel": "tf32x3_gemm_kernel (vvvv ladder + ring GEMMs)",
                     "achieved": kern_ach, "peak": gemm_peak, "unit": "TFLOP/s",
                     "frac": (kern_ach / gemm_peak) if kern_ach else None,
                     "traffic": gemm_traffic_60_240(),
                     "traffic_unit": "bytes per launch (mean of the vvvv and ring launches), DRAM read from "
                                     "small-case ncu captures scaled by pair tiles + C written once",
                     "peak_note": f"{peak_kind} bf16 {peaks['bf16_tflops']} TF/s / 2 (tf32 rate) / 3 (3xTF32)",
                     "launches_timed": nl.value},
        "clocks": clocks,
        "setup_s": setup_s,
    }

    out["hbm_kernels"] = hbm_kernels(plan, state["t"], diis, measured_peaks()[0]["hbm_gbs"])
    del diis, state
    torch.cuda.empty_cache()
    if not args.no_solve and rank == 0:
        # Full mixed solve (fresh amplitudes) + FP64 residual timing + a-posteriori FP64 check.
        params = dict(max_iterations=60, DIIS=True, e_convergence=1e-10, d_convergence=1e-8)
        hist = []
        torch.cuda.synchronize()
        ts = time.perf_counter()
        Em, tm = solve(plan, params, precision="mixed", history=hist)
        torch.cuda.synchronize()
        solve_s = time.perf_counter() - ts
        stats = hist[-1]
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record()
        r64 = plan.residual(tm, Em, _lib.PREC_FP64)
        f1.record()
        torch.cuda.synchronize()
        fp64_res_s = f0.elapsed_time(f1) / 1e3
        # amplitude correction implied by the FP64 residual at the mixed solution
        corr = plan.update(torch.zeros_like(tm), r64)
        max_corr = corr.abs().max().item()
        iters = len(hist) - 1
        out["solve"] = {
            "mixed_solve_s": solve_s, "E_mixed": [Em.real, Em.imag], "iterations": iters,
            "tf32_residuals": stats["tf32_residuals"], "fp64_residuals": stats["fp64_residuals"],
            "base_residual_s": stats.get("base_residual_s"),
            "iteration_s": [round(h["seconds"], 4) for h in hist[:-1]],
            "fp64_residual_s": fp64_res_s,
            "posterior_max_amplitude_correction": max_corr,
        }
        del r64, corr
        if not args.no_fp64_solve:
            # the plain FP64 GPU path (every GEMM on the FP64 pipe) solved to the same convergence
            # test from the same guess: measured wall time and the mixed solve's energy and
            # amplitude errors against it
            h64 = []
            torch.cuda.synchronize()
            ts = time.perf_counter()
            E64, t64 = solve(plan, params, precision="fp64", history=h64)
            torch.cuda.synchronize()
            fp64_s = time.perf_counter() - ts
            out["solve"].update({
                "fp64_solve_s": fp64_s, "E_fp64": [E64.real, E64.imag], "fp64_iterations": len(h64) - 1,
                "speedup_mixed_vs_fp64": fp64_s / solve_s,
                "abs_dE_mixed_vs_fp64": abs(Em - E64),
                "max_abs_amplitude_diff_mixed_vs_fp64": (tm - t64).abs().max().item(),
                "target": "|dE| <= 1e-9 Eh with the mixed solve faster than the FP64 solve"})
            del t64
        # Adjoint: one backward (CISD densities, vvvv block recomputed, 3xTF32 GEMMs) at the solution,
        # against the 2*(3N+3) = 24 full solves a finite-difference AAT/APT set needs for H2O (N = 3).
        from apyib_gb300.adjoint import densities
        torch.cuda.empty_cache()
        torch.cuda.synchronize()
        bwd = []
        for _ in range(2):    # the first call also pays the allocator's first-touch cost of its buffers
            a0 = time.perf_counter()
            Dm, Gm = densities(plan, tm, precision=_lib.PREC_TF32X3)
            torch.cuda.synchronize()
            bwd.append(time.perf_counter() - a0)
            if len(bwd) == 1:
                del Dm, Gm
        bwd_s = bwd[1]
        out["adjoint"] = {"backward_s": bwd_s, "backward_first_call_s": bwd[0], "fd_solves": 24,
                          "fd_estimate_s": 24 * solve_s,
                          "note": "one density backward vs 24 mixed solves (central differences, 3N+3 = 12 "
                                  f"parameters for H2O), both at o/v={o}/{v}"}
        del Dm, Gm, tm, plan
        torch.cuda.empty_cache()
        # Measured FP64-vs-mixed solve comparison where the FP64 solve fits the run: o/v = 40/160.
        o3, v3 = 40, 160
        prob3 = synthetic.so_factors(o3, v3, seed=0)
        eps3 = np.concatenate([np.repeat(prob3.eps_o, 2), np.repeat(prob3.eps_v, 2)])
        plan3 = CISDPlan(o3, v3, mixed=True)
        plan3.set_fock(torch.as_tensor(prob3.fock_so()), eps3)
        plan3.blocks_from_factors(torch.as_tensor(prob3.B), precision=_lib.PREC_OZAKI)
        it3, _, _ = mixed_iteration(plan3)
        c3_ms = timed_iterations(it3, 5, 3)
        res3 = {}
        for prec in ("fp64", "mixed"):
            h3 = []
            torch.cuda.synchronize()
            s0 = time.perf_counter()
            E3, _ = solve(plan3, params, precision=prec, history=h3)
            torch.cuda.synchronize()
            res3[prec] = (time.perf_counter() - s0, E3, len(h3) - 1)
        out["solve_40_160"] = {
            "fp64_solve_s": res3["fp64"][0], "mixed_solve_s": res3["mixed"][0],
            "speedup": res3["fp64"][0] / res3["mixed"][0],
            "abs_dE_mixed_vs_fp64": abs(res3["mixed"][1] - res3["fp64"][1]),
            "E_fp64": [res3["fp64"][1].real, res3["fp64"][1].imag],
            "iterations": {"fp64": res3["fp64"][2], "mixed": res3["mixed"][2]},
            "mixed_iteration_ms": c3_ms, "mixed_iteration_TFLOPs": alg_flops(o3, v3) / c3_ms / 1e9}
        del plan3, it3
    if not args.no_solve and rank == 0:
        out["ao_kernels_nbf150"] = ao_kernels(150)
        out["h2o_ccpvdz_bz"] = water_workloads()
    if not args.no_cpu and rank == 0:
        out["cpu_baseline"] = cpu_baseline_oracle(o, v)
        if "solve_40_160" in out:
            # the same comparison at o/v = 40/160: the GPU's mixed iteration against the
            # reference path's residual on the host cores (sampled the same way)
            c3 = cpu_baseline_oracle(40, 160, steps=2)
            g3 = out["solve_40_160"]["mixed_iteration_TFLOPs"]
            out["c3_40_160"] = {"gpu_mixed_iteration_TFLOPs": g3, "cpu_TFLOPs": c3["value"],
                                "cpu_full_residual_s_from_sample": c3["full_residual_s_from_sample"],
                                "cpu_sample": c3["sample"], "gpu_over_cpu": g3 / c3["value"]}
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
