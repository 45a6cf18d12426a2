"""Benchmark: Chebyshev (KPM) density of states at scale on one GB300.

Workload (one "step" = one full DoS solve): honeycomb lattice, 2 sites per
cell, nearest-neighbour t = -2.7, Anderson on-site disorder U[-0.5, 0.5]
(seed 1), 1024 x 1024 cells periodic (2,097,152 sites, 6.29M hoppings),
rescale bounds +-8.7 (|E| <= 3|t| + 0.5), M = 2048 Chebyshev moments, R = 32
random-phase vectors (e^{i theta}, seed 0), complex64 recursion with FP64
moment sums and Chebyshev doubling (bras = kets), Jackson kernel, rho(E) on
4096 energies reconstructed in FP64 on the device.

metric: site-moment-vector updates/s = N * M * R / step time.
  value : inputs resident in HBM (H~ and the kets block), device-timed.
  e2e   : the same solve through the C ABI drop-in (tbk_cheb_braket_real) with
          pinned HOST buffers: H~ CSC uploaded and compared with the cached
          plan's, kets read from host memory, moments read back, all inside
          the timed region of every call.
Also measured in the same run: the plain FP64 GPU path (complex128, one
moment per step, bras read every step — the reference's algorithm, fused),
the double-float plain path, the reference's own GPU algorithm (cuSPARSE
SpMM + cuBLAS dot per moment, restated in baseline/cusparse_kpm.cu), the CPU
oracle (the reference's CPU recursion restated in C, OpenMP over the random
vectors) on a bounded sample, full-size parity (all moments and rho against
the complex128 recursion), and one sub-record per other configuration
(`configs`: 1, 3, 5 and a shortened 4; configs 3 and 5 with the reference's
CPU Kubo path timed on bounded samples and extrapolated to one solve).

--impl reference: times the CPU restatement of the reference's KPM loop
(TB/numerical.h:363-381) on all host cores, on a bounded sample of the same
workload (the reference itself cannot be built: Eigen/FFTW/Spectra/C++23 are
absent), and prints the same JSON line with "impl": "reference".
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Chebyshev site-moment-vector updates/s vs FP64 plain; p50/p99 solve latency"
UNIT = "site-moment-vector updates/s"
L_CELLS = 1024
T_HOP = -2.7
W_DIS = 1.0            # U[-W/2, W/2] = U[-0.5, 0.5]
BOUND = 8.7
M_MOM = 2048
R_VEC = 32
N_E = 4096
WORKLOAD = ("KPM DoS: honeycomb 1024x1024 periodic (2,097,152 sites, nnz(H) 6.29M + 2.10M diag), "
            "t=-2.7, disorder U[-0.5,0.5] seed 1, M=2048, R=32 random-phase vectors seed 0, "
            "complex64 recursion + FP64 moments (doubling), Jackson kernel, rho(E) on 4096 energies")


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int, device=None) -> float:
    """The job's time: the maximum of every rank's value (all-reduce MAX over
    the default process group; the value itself at world size 1)."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, ws: int, steps: int, total_ms: float) -> float:
    """Whole-job throughput of weakly scaled replicas: every rank processes
    units_per_rank per step; the job takes the slowest rank's time."""
    return ws * units_per_rank * steps / (total_ms / 1e3)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(cp, ri, v, n, steps, threads, R=R_VEC):
    """Oracle recursion (plain path: one moment per step) on a bounded sample."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc

    kets = orc.random_phase_kets(n, R, 0)
    t0 = time.perf_counter()
    orc.cheb_moments(n, cp, ri, v, steps + 1, kets, kets, threads=threads, steps_limit=steps)
    dt = time.perf_counter() - t0
    return n * R * steps / dt, dt


def kubo_cpu_baseline(Ht, op, M, R, steps):
    """The reference's CPU Kubo path (TB/snippets.h:225-304 Greenwood, 306-456
    Bastin), timed on bounded samples of the same workload and extrapolated to
    one solve: per side M Chebyshev blocks of R vectors (Eigen's serial sparse
    x dense product: the oracle's C walk, 1 thread), one velocity product per
    block on the side that has an output operator plus one on an input side
    (TB/snippets.h:337-342), then mu_nm = L^H R over K = N R (Eigen's GEMM:
    here numpy's complex128 GEMM on all host threads, its rate measured on a
    256 x 65,536 x 256 product)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc

    cp, ri, v = Ht.to_csc()
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, R, 0)
    t0 = time.perf_counter()
    orc.cheb_blocks(n, cp, ri, v, steps + 1, kets)              # block 0 is the input: `steps` products
    t_step = (time.perf_counter() - t0) / steps
    ocp, ori, ov = op.to_csc()
    X = np.asfortranarray(kets)
    Y = np.zeros_like(X)
    t0 = time.perf_counter()
    orc.lib().tbo_csc_mult(n, orc._p(ocp), orc._p(ori), orc._p(np.ascontiguousarray(ov)), int(np.iscomplexobj(ov)),
                           R, orc._p(X), orc._p(Y))
    t_op = time.perf_counter() - t0
    rng = np.random.default_rng(0)
    A = rng.standard_normal((256, 65536)) + 1j * rng.standard_normal((256, 65536))
    B = rng.standard_normal((256, 65536)) + 1j * rng.standard_normal((256, 65536))
    dt = []
    for _ in range(2):
        t0 = time.perf_counter()
        A.conj() @ B.T
        dt.append(time.perf_counter() - t0)
    rate = 256 * 256 * 65536 / min(dt)                             # complex multiply-adds per second
    K = n * R
    recursion_s = 2 * M * t_step + (M + 1) * t_op
    gemm_s = M * M * K / rate
    return {"kind": "port", "value_s": recursion_s + gemm_s, "unit": "s per solve (extrapolated)",
            "recursion_s": recursion_s, "gemm_s": gemm_s,
            "recursion": {"cores": 1, "s_per_step": t_step, "steps_timed": steps, "operator_product_s": t_op},
            "gemm": {"cores": os.cpu_count(), "complex_macs_per_s": rate, "macs": M * M * K},
            "sample": "%d recursion steps and one velocity product of the workload's H~ (%d sites, R=%d), and a "
                      "256 x 65,536 x 256 complex128 GEMM; 2 M steps + (M + 1) products + M^2 N R MACs" %
                      (steps, n, R)}


def reference_gpu_algorithm(N, cp, ri, v, kets_ptr, R, n_mom):
    """The reference's own GPU algorithm (tight_binding/numerics_cuda.cu:190-255,
    restated in baseline/cusparse_kpm.cu): per call the CSC and the split Re / Im
    blocks are uploaded and the handles created; per moment two FP64 cuSPARSE
    SpMMs and two blocking cublasDdot traces.  Host CSC and kets in, moments out."""
    import ctypes as C

    lib = C.CDLL(str(ROOT / "baseline" / "_build" / "libref_cusparse.so"))
    fn = lib.ref_cusparse_braket_real
    fn.restype = C.c_int
    fn.argtypes = [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                   C.c_int32, C.c_void_p, C.c_void_p]
    mu = np.zeros(n_mom)
    t = np.zeros(2)
    rc = fn(N, len(ri), cp.ctypes.data, ri.ctypes.data, v.ctypes.data, n_mom, kets_ptr, kets_ptr, R, mu.ctypes.data,
            t.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"reference cuSPARSE path failed at baseline/cusparse_kpm.cu:{rc}")
    return mu, float(t[0]), float(t[1])


def build_host_system():
    """The rescaled H~ of the workload as host CSC arrays (built on the device)."""
    import tight_binding_gb300 as tb

    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, T_HOP), (L_CELLS, L_CELLS))
    X.set_scalar_disorder(W_DIS, 1)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    G = tb.GreenFunction(M_MOM, H, -BOUND, BOUND)
    return X, H, G


def oracle_system():
    """Same H~ built by the CPU oracle (reference arm: no GPU involved)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc

    s3 = np.sqrt(3.0)
    bases = np.array([[1.5, -s3 / 2, 0], [1.5, s3 / 2, 0]]).T
    pos = np.array([[0, 0, 0], [1, 0, 0.0]])
    # canonical table of Honeycomb + add_hopping("A", 1NN, t) + set_scalar_field zeros
    hf = [1, 1, 1, 0, 1]
    ht = [0, 0, 0, 0, 1]
    hv = [[1, 0, 0], [0, 1, 0], [0, 0, 0], [0, 0, 0], [0, 0, 0]]
    tt = [T_HOP, T_HOP, T_HOP, 0.0, 0.0]
    N = 2 * L_CELLS * L_CELLS
    V = orc.uniform_disorder(N, W_DIS, 1)
    spec = orc.LatticeSpec(2, [L_CELLS, L_CELLS], bases, pos, hf, ht, hv, tt, mode=orc.MODE_PERIODIC_BARE,
                           is_complex=False, extend=[1, 1], scalar_site=V)
    cp, ri, v = orc.build_csc(spec)
    ocp, ori, ov = orc.rescale_csc(N, cp, ri, v, BOUND, 0.0)
    return N, ocp, ori, ov


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    N, cp, ri, v = oracle_system()
    steps_per_sample = args.cpu_steps
    if args.warmup > 0:
        cpu_sample(cp, ri, v, N, 1, threads)
    vals, times = [], []
    for _ in range(args.steps):
        r, dt = cpu_sample(cp, ri, v, N, steps_per_sample, threads)
        vals.append(r)
        times.append(dt)
    value = float(np.mean(vals))
    sample = (f"{steps_per_sample} recursion steps (one moment each) of the workload's H~ x 32 vectors per "
              f"step, C restatement of TB/numerical.h:363-381, OpenMP over vectors")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sites": N, "moments": M_MOM, "vectors": R_VEC},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import torch

    import tight_binding_gb300 as tb
    from tight_binding_gb300 import capi

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    X, H, G = build_host_system()
    Ht = G.scaled_HE
    N = Ht.shape[0]
    # resident inputs: kets block (Eigen layout N x R column-major complex128)
    kets_h = tb.bases_of_uniform_ampl_with_random_phases(N, R_VEC, 0 + rank)
    kets_d = torch.from_numpy(np.ascontiguousarray(kets_h.T)).to(dev)        # (R, N) row-major == N x R col-major
    mu_d = torch.zeros(M_MOM, dtype=torch.float64, device=dev)
    solver = tb.KpmSolver(Ht, R_VEC, precision="mixed", doubling=True, flags=capi.FLAG_DEVICE_PTRS)
    E = np.cos((np.arange(N_E) + 0.5) * np.pi / N_E) * 0.999
    jack = tb.Jackson()

    def step():
        with torch.cuda.stream(stream):
            solver.run_device(M_MOM, kets_d.data_ptr(), kets_d.data_ptr(), mu_d.data_ptr(), sh)
            mu = mu_d.cpu().numpy()
        rho = tb.dos_from_moments(mu, jack, R_VEC, E)
        return mu, rho

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    rec_ms, rec_launch, rec_bytes = [], 0, 0.0
    torch.cuda.synchronize()
    ev[0].record(stream)
    for k in range(args.steps):
        mu, rho = step()
        ev[k + 1].record(stream)
        ms, nl, b = solver.last_timing()
        rec_ms.append(ms)
        rec_launch, rec_bytes = nl, b
    torch.cuda.synchronize()
    clocks = sampler.stop()
    per_step = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    total_ms = max_over_ranks(total_ms, ws, dev)
    updates = float(N) * M_MOM * R_VEC
    value = job_rate(updates, ws, args.steps, total_ms)

    if rank != 0:
        if ws > 1:
            dist.barrier()
            dist.destroy_process_group()
        return 0

    # ---- roofline of the recursion kernel (live CUDA events on the launching stream)
    peak, peak_kind = peaks()
    avg_launch_ms = float(np.mean(rec_ms)) / rec_launch
    achieved = rec_bytes / (avg_launch_ms / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "kpm_step_traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get("bytes_per_launch")
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "kernel": "kpm_step_kernel<float,32,real,doubling>", "launches_per_step": rec_launch,
                "algorithmic_bytes_per_launch": rec_bytes, "avg_launch_us": avg_launch_ms * 1e3}

    # ---- e2e through the C-ABI drop-in with pinned host buffers
    cp, ri, v = Ht.to_csc()
    cp_p = torch.from_numpy(cp).pin_memory()
    ri_p = torch.from_numpy(ri).pin_memory()
    v_p = torch.from_numpy(v).pin_memory()
    kets_p = torch.from_numpy(np.ascontiguousarray(kets_h.T)).pin_memory()
    mu_h = torch.zeros(M_MOM, dtype=torch.float64).pin_memory()
    h2d = cp_p.numel() * 4 + ri_p.numel() * 4 + v_p.numel() * 8 + kets_p.numel() * 16
    d2h = M_MOM * 8
    flags = capi.PREC_MIXED | capi.FLAG_DOUBLING

    def e2e_call():
        kp = kets_p.data_ptr()
        capi.check(capi.lib().tbk_cheb_braket_real(N, ri_p.numel(), cp_p.data_ptr(), ri_p.data_ptr(), v_p.data_ptr(),
                                                  M_MOM, kp, kp, R_VEC, flags, mu_h.data_ptr()))

    e2e_call()
    e2e_steps = max(3, min(args.steps, 5))
    call_ms = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        e2e_call()
        call_ms.append((time.perf_counter() - t1) * 1e3)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": updates / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "ms_per_step": e2e_s * 1e3, "calls_ms": call_ms,
           "api": "tbk_cheb_braket_real (drop-in for cuda::Cheb_first_kind_seq_braket; plan cached across calls, "
                  "CSC and kets uploaded and compared every call)"}
    e2e_err = float(np.max(np.abs(mu_h.numpy() - mu)) / abs(mu[0]))

    # ---- plain FP64 GPU path (reference algorithm, fused): one moment per step, bras read each step
    fp = tb.KpmSolver(Ht, R_VEC, precision="fp64", doubling=False, flags=capi.FLAG_DEVICE_PTRS)
    m64 = args.fp64_moments
    mu64_d = torch.zeros(m64, dtype=torch.float64, device=dev)
    with torch.cuda.stream(stream):
        fp.run_device(m64, kets_d.data_ptr(), kets_d.data_ptr(), mu64_d.data_ptr(), sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    with torch.cuda.stream(stream):
        fp.run_device(m64, kets_d.data_ptr(), kets_d.data_ptr(), mu64_d.data_ptr(), sh)
    e1.record(stream)
    torch.cuda.synchronize()
    fp_ms = e0.elapsed_time(e1)
    fp_value = float(N) * m64 * R_VEC / (fp_ms / 1e3)
    mu64 = mu64_d.cpu().numpy()
    mixed_vs_fp64 = float(np.max(np.abs(mu[:m64] - mu64)) / abs(mu64[0]))
    ms64, nl64, b64 = fp.last_timing()
    del fp

    # ---- the reference's GPU algorithm itself (cuSPARSE + cuBLAS per moment), same H~, kets and moments
    ref_mu, ref_call_ms, ref_loop_ms = reference_gpu_algorithm(N, cp, ri, v, kets_p.data_ptr(), R_VEC, m64)
    units64 = float(N) * m64 * R_VEC
    reference_gpu = {
        "algorithm": "tight_binding/numerics_cuda.cu:190-255 restated (baseline/cusparse_kpm.cu): per moment 2 FP64 "
                     "cusparseSpMM (CSC, Re/Im blocks) + 2 blocking cublasDdot; CSC, blocks and handles per call",
        "moments": m64, "call_ms": ref_call_ms, "loop_ms": ref_loop_ms,
        "value_call": units64 / (ref_call_ms / 1e3), "value_loop": units64 / (ref_loop_ms / 1e3), "unit": UNIT,
        "rel_err_vs_fp64_plain": float(np.max(np.abs(ref_mu - mu64)) / abs(mu64[0])),
        "speedup_fp64_plain_over_it": ref_loop_ms / fp_ms,
    }

    # ---- double-float plain path: the same algorithm with FP64-class accuracy on the FP32 pipe
    ddp = tb.KpmSolver(Ht, R_VEC, precision="dd", doubling=False, flags=capi.FLAG_DEVICE_PTRS)
    with torch.cuda.stream(stream):
        ddp.run_device(m64, kets_d.data_ptr(), kets_d.data_ptr(), mu64_d.data_ptr(), sh)
    torch.cuda.synchronize()
    e0.record(stream)
    with torch.cuda.stream(stream):
        ddp.run_device(m64, kets_d.data_ptr(), kets_d.data_ptr(), mu64_d.data_ptr(), sh)
    e1.record(stream)
    torch.cuda.synchronize()
    dd_ms = e0.elapsed_time(e1)
    mudd = mu64_d.cpu().numpy()
    msdd, nldd, bdd = ddp.last_timing()
    del ddp

    # ---- full-size parity: all M_MOM moments and rho on the N_E energies against
    # the complex128 (FP64) recursion of the same resident kets (doubling)
    fpd = tb.KpmSolver(Ht, R_VEC, precision="fp64", doubling=True, flags=capi.FLAG_DEVICE_PTRS)
    mu_full_d = torch.zeros(M_MOM, dtype=torch.float64, device=dev)
    with torch.cuda.stream(stream):
        fpd.run_device(M_MOM, kets_d.data_ptr(), kets_d.data_ptr(), mu_full_d.data_ptr(), sh)
    torch.cuda.synchronize()
    mu_ref = mu_full_d.cpu().numpy()
    del fpd
    d_mu = np.abs(mu - mu_ref) / abs(mu_ref[0])
    rho_ref = tb.dos_from_moments(mu_ref, jack, R_VEC, E)
    full_parity = {"reference": "complex128 recursion (FP64), same kets, doubling",
                   "max_rel_mu_all_moments": float(d_mu.max()),
                   "max_rel_mu_per_256": [float(d_mu[i:i + 256].max()) for i in range(0, M_MOM, 256)],
                   "max_rel_rho": float(np.max(np.abs(rho - rho_ref)) / np.max(rho_ref)),
                   "bound": 1e-5}

    # ---- CPU baseline: oracle on a bounded sample (all host cores)
    threads = os.cpu_count() or 1
    cpu_val, cpu_dt = cpu_sample(cp, ri, v, N, args.cpu_steps, threads)
    one_steps = max(2, args.cpu_steps // 16)
    one_val, one_dt = cpu_sample(cp, ri, v, N, one_steps, 1)
    cpu = {"value": cpu_val, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{args.cpu_steps} recursion steps x 32 vectors of the same H~ ({cpu_dt:.1f} s), "
                     f"C restatement of TB/numerical.h:363-381, OpenMP over vectors",
           "single_thread": {"value": one_val, "cores": 1, "sample": f"{one_steps} steps x 32 vectors ({one_dt:.1f} s), "
                             "the serial product the reference's Eigen path runs"}}

    launches_per_step = 1 + rec_launch + 2 + 2     # load kets, recursion, reduce+assemble, kernel+rho
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sites": int(N), "moments": M_MOM, "vectors": R_VEC},
        "config_details": {"nnz_Ht": int(Ht.nnz), "energies": N_E,
                           "precision": "complex64 recursion, FP64 moment sums, doubling",
                           "parallelism": "replicas" if ws > 1 else "single GPU",
                           "l2": "inputs larger than L2 (537 MB vector block per step, 129 MB L2); no flush"},
        "latency_ms": {"p50": float(np.percentile(per_step, 50)), "p99": float(np.percentile(per_step, 99))},
        "e2e": e2e, "gpu_launches": launches_per_step * args.steps,
        "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
        "fp64_plain": {"value": fp_value, "unit": UNIT, "moments": m64, "ms": fp_ms,
                       "kernel_ms": ms64, "launches": nl64, "bytes_per_launch": b64,
                       "speedup_mixed_over_fp64": value / fp_value},
        "reference_gpu": dict(reference_gpu, speedup_mixed_over_it=value / reference_gpu["value_loop"],
                              speedup_dd_plain_over_it=ref_loop_ms / dd_ms),
        "dd_plain": {"value": float(N) * m64 * R_VEC / (dd_ms / 1e3), "unit": UNIT, "moments": m64, "ms": dd_ms,
                     "kernel_GBps": bdd * nldd / (msdd / 1e3) / 1e9, "speedup_over_fp64_plain": fp_ms / dd_ms,
                     "rel_err_vs_fp64": float(np.max(np.abs(mudd - mu64)) / abs(mu64[0]))},
        "parity": {"mixed_vs_fp64_rel_err_first_%d_moments" % m64: mixed_vs_fp64, "e2e_vs_resident_rel": e2e_err,
                   "full": full_parity},
    }
    if not args.no_configs:
        line["configs"] = other_configs(args)
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def other_configs(args):
    """The other configurations, one sub-record each, measured in the same run:
    config 1 (square 64^2 DoS latency, drop-in and resident), config 3
    (Kubo-Bastin sigma_xy with its FP64-reference parity), config 5
    (Kubo-Greenwood sigma_xx, FCC 128^3) and config 4 shortened to
    --serve-requests-default requests of the same arrival process.  A failing
    leg records its error instead of ending the run."""
    import types

    out = {}

    def leg(name, fn):
        t0 = time.perf_counter()
        try:
            out[name] = fn()
        except Exception as e:                 # recorded, not raised: the main line stands
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["leg_wall_s"] = time.perf_counter() - t0

    small = types.SimpleNamespace(steps=50, warmup=3)
    leg("c1_square64_dos", lambda: run_small(small))
    leg("c3_kubo_bastin_sigma_xy", lambda: run_kubo(3, parity=True))
    leg("c5_kubo_greenwood_sigma_xx", lambda: run_kubo(5))
    sv = types.SimpleNamespace(serve_requests=args.serve_requests_default, serve_gap_ms=args.serve_gap_ms,
                               serve_precision="mixed", serve_budget_gb=args.serve_budget_gb,
                               serve_round=args.serve_round, serve_step_gb=args.serve_step_gb)
    leg("c4_serving_stream", lambda: serve_line(sv))
    return out


def peaks_tensor():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        # TF32 dense rate is half the BF16 rate on this part; reported against half the measured cuBLAS BF16 burst
        return float(d["bf16_tflops"]) / 2.0, "half of measured bf16 burst (TF32 = BF16/2)"
    return 1900.0 / 2.0, "half of fallback bf16"


def run_kubo(config: int, tensor: bool = True, recursion: str = "mixed", fuse_ops: bool = False, moments: int = 0,
             budget_gb: float = 0.0, parity: bool = False, cpu: bool = True):
    """Kubo legs: config 3 (Bastin sigma_xy, square 256^2 open-x / periodic-y, Landau
    flux 1/64, M = 512, R = 16, seed 2) or config 5 (Greenwood sigma_xx, FCC 128^3
    periodic, on-site U[-1,1] seed 4, M = 1024, R = 8).  parity (config 3): also
    the FP64 reference form (complex128 recursion and blocks, FP64 GEMM) on the
    same seeded vectors, and max |d sigma_xy| / max |sigma_xy| against it.
    cpu: the reference's CPU path on bounded samples, extrapolated
    (kubo_cpu_baseline)."""
    import tight_binding_gb300 as tb

    sig = {}

    def once():
        t0 = time.perf_counter()
        if config == 3:
            L, M, R = 256, moments or 512, 16
            X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (L, L))
            G = np.zeros((3, 3))
            G[1, 0] = 2 * np.pi / 64
            X.set_gauge_linear(G, np.zeros(3))
            H = X.get_Hamiltonian_periodic_extend_bare_sparse([0, 1], complex)
            out = tb.conductivity_Kubo_Bastin(H, X.op_position(0), X.op_position(1), M, -4.0, 4.0, R=R, seed=2,
                                              tensor=tensor, recursion=recursion, fuse_ops=fuse_ops, budget_gb=budget_gb)
            result = {"E_F_points": int(len(out["E"])), "sigma_xy_at_E0": float(out["sigma_re"][len(out["E"]) // 2])}
            sig["args"] = (H, X.op_position(0), X.op_position(1), M, -4.0, 4.0)
            sig["R"] = R
            sig["cpu"] = (H, X.op_position(1), M, R, -4.0, 4.0, 16)        # input side: v_y r
            sig["sigma"] = out["sigma_re"]
            workload = "Kubo-Bastin sigma_xy: square 256x256 open-x/periodic-y, Landau flux 1/64, M=512, R=16 seed 2"
        else:
            L, M, R = 128, moments or 1024, 8
            X = tb.PartialLattice(tb.FCC().add_hopping("A", 1, 1.0), (L, L, L))
            X.set_scalar_disorder(2.0, 4)
            H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1, 1], complex)
            eps, sigma, mu = tb.conductivity_spectrum(H, X.op_position(0), X.op_position(1), M, R=R, seed=4,
                                                      E_min=-13.0, E_max=13.0, tensor=tensor, recursion=recursion,
                                                      fuse_ops=fuse_ops, budget_gb=budget_gb)
            result = {"energies": int(len(eps)), "sigma_xx_max": float(np.max(sigma))}
            sig["cpu"] = (H, X.op_position(0), M, R, -13.0, 13.0, 2)
            workload = "Kubo-Greenwood sigma_xx: FCC 128^3 periodic, disorder U[-1,1] seed 4, M=1024, R=8"
        return time.perf_counter() - t0, workload, result

    # the first call includes CUDA context creation and module loading; the
    # second is the steady-state cost of a solve
    wall_cold, workload, result = once()
    wall, workload, result = once()

    tmg = tb.kubo_last_timing()
    peak, src = peaks_tensor()
    useful = tmg["gemm_flops"] / (3.0 if tensor else 1.0)       # one complex GEMM = 8 M^2 K real flops
    line = {"workload": workload, "path": "tcgen05 3xTF32" if tensor else "CUDA-core FP32", "recursion": recursion,
            "fused_operator_products": fuse_ops, "moments": moments or (512 if config == 3 else 1024),
            "wall_s": wall, "wall_cold_s": wall_cold, "blocks_ms": tmg["ms_blocks"], "gemm_ms": tmg["ms_gemm"],
            "chunks": tmg["chunks"],
            "gemm_tflops_issued": tmg["gemm_flops"] / (tmg["ms_gemm"] / 1e3) / 1e12,
            "gemm_tflops_useful": useful / (tmg["ms_gemm"] / 1e3) / 1e12,
            "tensor_peak_tflops": peak, "tensor_peak_source": src,
            "blocks_GBps": tmg["block_bytes"] / (tmg["ms_blocks"] / 1e3) / 1e9, **result}
    hbm, hbm_src = peaks()
    line["blocks_roofline"] = {"bound": "hbm", "achieved": line["blocks_GBps"], "peak": hbm, "unit": "GB/s",
                               "frac": line["blocks_GBps"] / hbm, "peak_source": hbm_src,
                               "bytes": "algorithmic: work vectors + matrix per pass + complex64 stores"}
    if tensor:
        line["tensor_util"] = line["gemm_tflops_issued"] / peak
    if cpu:
        H, pos, M_c, R_c, lo, hi, steps = sig["cpu"]
        Ht = tb.GreenFunction(M_c, H, lo, hi).scaled_HE
        cb = kubo_cpu_baseline(Ht, tb.commutator(Ht, pos), M_c, R_c, steps)
        cb["speedup_vs_wall"] = cb["value_s"] / wall
        line["cpu_baseline"] = cb
    if parity and config == 3:
        t0 = time.perf_counter()
        ref = tb.conductivity_Kubo_Bastin(*sig["args"], R=sig["R"], seed=2, recursion="fp64", fp64_blocks=True)
        line["parity"] = {"reference": "FP64 form: complex128 recursion and stored blocks, FP64 CUDA-core GEMM",
                          "max_rel_sigma_xy": float(np.max(np.abs(sig["sigma"] - ref["sigma_re"])) /
                                                    np.max(np.abs(ref["sigma_re"]))),
                          "bound": 1e-5, "reference_s": time.perf_counter() - t0}
    return line


SERVE_KINDS = ("square", "honeycomb", "kagome", "lieb", "fcc")


def serve_stream(n: int, gap_ms: float, seed: int = 3):
    """The serving workload: Poisson arrivals (mean gap gap_ms), lattice kind
    uniform over SERVE_KINDS, linear size U{32..512} (2D) or U{16..64} (FCC),
    disorder W ~ U[0, 2], M in {256, 512, 1024}, R in {4, 8, 16, 32, 64}."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(gap_ms, n)
    arrive = np.cumsum(gaps) - gaps[0]
    kind = rng.integers(0, len(SERVE_KINDS), n)
    L2 = rng.integers(32, 513, n)
    L3 = rng.integers(16, 65, n)
    W = rng.uniform(0.0, 2.0, n)
    M = rng.choice([256, 512, 1024], n)
    R = rng.choice([4, 8, 16, 32, 64], n)
    out = []
    for i in range(n):
        k = SERVE_KINDS[kind[i]]
        out.append(dict(t_ms=float(arrive[i]), kind=k, L=int(L3[i] if k == "fcc" else L2[i]), W=float(W[i]),
                        M=int(M[i]), R=int(R[i]), seed=i))
    return out


def run_serve(args):
    """Config 4: a stream of DoS requests through the continuous-batching server
    (admission under the HBM budget, graph-captured rounds packed over all
    running requests).  value = requests/s over the whole stream; latency =
    submit -> result per request."""
    line = serve_line(args)
    if dist_info()[1] == 0:
        print(json.dumps(line), flush=True)
    return 0


def serve_line(args):
    import tight_binding_gb300 as tb
    from tight_binding_gb300.serving import model_bounds, model_cell

    ws, rank, local = dist_info()
    reqs = serve_stream(args.serve_requests, args.serve_gap_ms)
    # weak scaling over ranks: rank r serves requests r, r + ws, ...
    mine = reqs[rank::ws]
    cells = {k: model_cell(k) for k in SERVE_KINDS}
    srv = tb.DosServer(budget_gb=args.serve_budget_gb, steps_per_round=args.serve_round, autotune=True,
                       step_gb=args.serve_step_gb)
    tuning = srv.tuning()
    tickets = [None] * len(mine)
    ready = threading.Semaphore(0)
    err = []

    def lat(q):
        span = (q["L"],) * (3 if q["kind"] == "fcc" else 2)
        X = tb.PartialLattice(cells[q["kind"]], span)
        if q["W"] > 0:
            X.set_scalar_disorder(q["W"], q["seed"])
        return X

    def submitter():
        t0 = time.perf_counter()
        try:
            for i, q in enumerate(mine):
                dt = q["t_ms"] / 1e3 - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                emin, emax = model_bounds(q["kind"], q["W"])
                tickets[i] = srv.submit(lat(q), q["M"], q["R"], seed=q["seed"], e_min=emin, e_max=emax,
                                        precision=args.serve_precision)
                ready.release()
        except Exception as e:          # surfaced by the main thread
            err.append(e)
            ready.release()

    sampler = ClockSampler(local)
    sampler.start()
    t_start = time.perf_counter()
    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    lat_ms, queued_ms, build_ms, bad = [], [], [], 0
    for i in range(len(mine)):
        ready.acquire()
        if err:
            raise err[0]
        mu, times = srv.result(tickets[i], timeout_s=1800)
        q = mine[i]
        if not (np.all(np.isfinite(mu)) and abs(mu[0] - q["R"]) < 1e-3 * q["R"]):
            bad += 1
        lat_ms.append(times[3])
        queued_ms.append(times[0])
        build_ms.append(times[1])
    wall = time.perf_counter() - t_start
    th.join()
    clocks = sampler.stop()
    st = srv.stats()
    srv.close()
    peak, peak_kind = peaks()
    achieved = st["bytes"] / (st["busy_ms"] / 1e3) / 1e9 if st["busy_ms"] > 0 else 0.0
    line = {
        "metric": "DoS serving stream: requests/s and p50/p99 latency (submit -> moments)",
        "value": len(mine) / wall, "unit": "requests/s",
        "n_gpus": ws, "steps": len(mine), "warmup": 0, "ms_per_step": 1e3 * wall / len(mine),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"mixed": "c64", "fp64": "c128", "dd": "double-float c128"}[args.serve_precision],
        "data": "synthetic",
        "config": {"workload": f"{args.serve_requests} DoS requests, Poisson arrivals mean gap "
                               f"{args.serve_gap_ms} ms (seed 3); square/honeycomb/Kagome/Lieb L~U{{32..512}}, "
                               f"FCC L~U{{16..64}}; NN t=1.0 + disorder W~U[0,2]; M in {{256,512,1024}}; "
                               f"R in {{4,8,16,32,64}}; {args.serve_precision} recursion (doubling)",
                   "budget_gb": args.serve_budget_gb, "steps_per_round": args.serve_round,
                   "step_gb": args.serve_step_gb, "l2": "resident working set far above L2; no flush"},
        "updates_per_s": st["updates"] / wall,
        "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                       "mean": float(np.mean(lat_ms)), "max": float(np.max(lat_ms)),
                       "queued_p50": float(np.percentile(queued_ms, 50)),
                       "build_p50": float(np.percentile(build_ms, 50))},
        "wall_s": wall, "gpu_busy_frac": st["busy_ms"] / 1e3 / wall,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel": "srv_step_kernel (all groups, over GPU-busy time)"},
        "gpu_launches": int(st["launches"]), "server": st, "tuning": tuning, "bad_results": bad, "clocks": clocks,
    }
    return line


def run_serve_single(args):
    """Profiling case of the serving step kernel: one honeycomb --cells^2 request
    (t = 1, disorder W = 1 seed 1, R = 32, M = --moments, mixed) through a server
    (launch-shape tuner on unless --serve-no-tune), twice; reports the second's
    HBM rate."""
    import tight_binding_gb300 as tb
    from tight_binding_gb300.serving import model_bounds, model_cell

    srv = tb.DosServer(autotune=not args.serve_no_tune)
    X = tb.PartialLattice(model_cell("honeycomb"), (args.cells, args.cells))
    X.set_scalar_disorder(1.0, 1)
    lo, hi = model_bounds("honeycomb", 1.0)
    for _ in range(2):
        b0 = srv.stats()
        mu, t = srv.result(srv.submit(X, args.moments, R_VEC, seed=0, e_min=lo, e_max=hi))
        b1 = srv.stats()
    gbs = (b1["bytes"] - b0["bytes"]) / ((b1["busy_ms"] - b0["busy_ms"]) / 1e3) / 1e9
    print(json.dumps({"serve_single": f"honeycomb {args.cells}^2", "sites": X.get_total_number(),
                      "moments": args.moments, "GBps": gbs, "rounds": b1["rounds"] - b0["rounds"],
                      "busy_ms": b1["busy_ms"] - b0["busy_ms"], "mu0": float(mu[0])}), flush=True)
    srv.close()
    return 0


def run_gemm(args):
    """mu_nm GEMM alone on seeded random complex blocks (M x K each, rounded to
    complex64 on the device): the profiling case of the tensor-core kernel."""
    import tight_binding_gb300 as tb

    M, K = args.gemm
    rng = np.random.default_rng(M + K)
    L = (rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))) / np.sqrt(K)
    R = (rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))) / np.sqrt(K)
    tensor = not args.cuda_core_mu
    for _ in range(2):
        tb.mu_from_blocks(L, R, tensor=tensor)
    t = tb.kubo_last_timing()
    peak, src = peaks_tensor()
    issued = t["gemm_flops"] / (t["ms_gemm"] / 1e3) / 1e12
    print(json.dumps({"gemm": [M, K], "path": "tcgen05 3xTF32" if tensor else "CUDA-core FP32", "ms": t["ms_gemm"],
                      "tflops_issued": issued, "tensor_util": issued / peak if tensor else None,
                      "peak_source": src}), flush=True)
    return 0


def run_expand(args):
    """exp(-i H t) applied to R = 8 random-phase vectors on the benchmark
    honeycomb (--cells^2 cells, disorder seed 1) through tbk_cheb_expand, in
    --precision, host vectors in and out (end to end, wall clock).  Algorithmic
    bytes per term (one Clenshaw step): H~ once (ELL off-diagonal index +
    value, diagonal value) and four vector streams (b_{k+1} gathered, b_{k+2}
    read, b_k written, the kets read for the c_k term)."""
    import tight_binding_gb300 as tb

    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, T_HOP), (args.cells, args.cells))
    X.set_scalar_disorder(W_DIS, 1)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    G = tb.GreenFunction(16, H, -BOUND, BOUND)
    n = H.shape[0]
    R = 8
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, R, 0)
    coef = tb.evolution_coefficients(G.a, G.b, args.expand)
    tb.cheb_expand(G.scaled_HE, coef[:4], kets, args.precision)          # warm-up (ELL, modules)
    t0 = time.perf_counter()
    out = tb.cheb_expand(G.scaled_HE, coef, kets, args.precision)
    dt = time.perf_counter() - t0
    csz = {"mixed": 8, "fp64": 16, "dd": 16}[args.precision]      # complex element: c64, c128, 2 x (hi, lo) float
    vsz = {"mixed": 4, "fp64": 8, "dd": 8}[args.precision]        # real matrix value
    nnz_off = 3 * n
    per_term = nnz_off * (4 + vsz) + n * vsz + n * R * 4 * csz
    print(json.dumps({"expand": "exp(-iHt)", "t": args.expand, "terms": len(coef), "sites": n, "R": R,
                      "precision": args.precision, "s_e2e": dt,
                      "updates_per_s": n * R * len(coef) / dt, "GBps_e2e": per_term * len(coef) / dt / 1e9,
                      "norm_err": float(np.max(np.abs(np.linalg.norm(out, axis=0) - 1.0)))}), flush=True)
    return 0


def run_small(args):
    """Config-1 DoS (the reference's CPU-sized case): square 64 x 64 periodic,
    t = 1, H~ = H / 4.05, M = 256, R = 8 random-phase vectors (seed 0), Jackson
    kernel, rho on 1,024 energies in [-4, 4].  Launch/latency bound (a 512 KB
    vector block): reports per-solve latency p50/p99 over --steps solves of the
    resident plan (FP64, mixed and double-float, doubling; per-step launches
    replayed as a CUDA graph, without the graph, and the opt-in one-launch
    recursion: one CTA per vector where H~ has row classes and a complex64 or
    double-float vector fits one SM, else a cluster per vector), the
    drop-in C-ABI call with host buffers (H~ uploaded every call, as the
    reference's cuSPARSE path does), and the CPU oracle on the whole solve."""
    import torch

    import tight_binding_gb300 as tb
    from tight_binding_gb300 import capi

    L, M, R, NE = 64, 256, 8, 1024
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (L, L))
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    G = tb.GreenFunction(M, H, -4.05, 4.05)
    Ht = G.scaled_HE
    N = Ht.shape[0]
    kets_h = tb.bases_of_uniform_ampl_with_random_phases(N, R, 0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    kets_d = torch.from_numpy(np.ascontiguousarray(kets_h.T)).to(dev)
    mu_d = torch.zeros(M, dtype=torch.float64, device=dev)
    E = np.linspace(-4.0, 4.0, NE) / 4.05 * 0.999
    steps = max(args.steps, 50)
    out = {"small_dos": "square 64x64 PBC, t=1, a=4.05, M=256, R=8, Jackson, 1024 energies", "sites": N,
           "solves": steps}
    ref_mu = None
    for name, prec, extra in (("fp64", "fp64", 0), ("fp64_no_graph", "fp64", capi.FLAG_NO_GRAPH),
                              ("fp64_one_launch", "fp64", capi.FLAG_PERSISTENT), ("mixed", "mixed", 0),
                              ("mixed_one_launch", "mixed", capi.FLAG_PERSISTENT),
                              ("mixed_two_step", "mixed", capi.FLAG_TWO_STEP), ("dd", "dd", 0),
                              ("dd_one_launch", "dd", capi.FLAG_PERSISTENT)):
        sol = tb.KpmSolver(Ht, R, precision=prec, doubling=True, flags=capi.FLAG_DEVICE_PTRS | extra)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * steps)]
        for _ in range(args.warmup + 2):
            with torch.cuda.stream(stream):
                sol.run_device(M, kets_d.data_ptr(), kets_d.data_ptr(), mu_d.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        for k in range(steps):
            ev[2 * k].record(stream)
            with torch.cuda.stream(stream):
                sol.run_device(M, kets_d.data_ptr(), kets_d.data_ptr(), mu_d.data_ptr(), stream.cuda_stream)
            ev[2 * k + 1].record(stream)
        torch.cuda.synchronize()
        lat = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(steps)]
        mu = mu_d.cpu().numpy()
        if ref_mu is None:
            ref_mu = mu.copy()
        out[name] = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                     "updates_per_s": N * M * R / (float(np.percentile(lat, 50)) / 1e3),
                     "rel_err_vs_fp64": float(np.max(np.abs(mu - ref_mu)) / abs(ref_mu[0]))}
        del sol
    # drop-in C-ABI call with host buffers (upload of H~ and kets, read-back of mu)
    cp, ri, v = Ht.to_csc()
    kets_c = np.asfortranarray(kets_h)
    mu_h = np.zeros(M)
    flags = capi.PREC_FP64 | capi.FLAG_DOUBLING

    def dropin():
        capi.check(capi.lib().tbk_cheb_braket_real(N, len(ri), capi.ptr(cp), capi.ptr(ri), capi.ptr(v), M,
                                                   capi.ptr(kets_c), capi.ptr(kets_c), R, flags, capi.ptr(mu_h)))

    for _ in range(args.warmup):
        dropin()
    t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        dropin()
        t.append((time.perf_counter() - t0) * 1e3)
    out["dropin_e2e"] = {"p50_ms": float(np.percentile(t, 50)), "p99_ms": float(np.percentile(t, 99)),
                         "rel_err_vs_fp64": float(np.max(np.abs(mu_h - ref_mu)) / abs(ref_mu[0]))}
    # reconstruction of rho on the 1,024 energies
    t0 = time.perf_counter()
    rho = tb.dos_from_moments(ref_mu, tb.Jackson(), R, E)
    out["rho_ms"] = (time.perf_counter() - t0) * 1e3
    out["rho_integral"] = float(np.trapezoid(rho, E)) if hasattr(np, "trapezoid") else None
    # CPU oracle on the whole solve (plain path, one moment per step)
    for threads in (1, os.cpu_count() or 1):
        rate, dt = cpu_sample(cp, ri, v, N, M - 1, threads, R)
        out[f"cpu_oracle_{threads}t"] = {"ms": dt * 1e3, "updates_per_s": rate}
    return out


def run_kernel_only(args):
    """Small case of the same kernel for ncu captures: one mixed-precision DoS
    solve (doubling) on a honeycomb of --cells^2 cells, R = 32."""
    import tight_binding_gb300 as tb

    cell = tb.Honeycomb()
    if not args.no_hopping:
        cell.add_hopping("A", 1, T_HOP)
    X = tb.PartialLattice(cell, (args.cells, args.cells))
    X.set_scalar_disorder(W_DIS, 1)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    G = tb.GreenFunction(args.moments, H, -BOUND, BOUND)
    from tight_binding_gb300 import capi

    flags = (capi.FLAG_STAGED if args.staged else 0) | (capi.FLAG_TWO_STEP if args.two_step else 0)
    s = tb.KpmSolver(G.scaled_HE, R_VEC, precision=args.precision, doubling=args.precision == "mixed", flags=flags)
    for _ in range(2):
        mu = s.run_random(args.moments, 0)
    ms, nl, b = s.last_timing()
    print(json.dumps({"staged": args.staged, "two_step": args.two_step, "no_hopping": args.no_hopping, "precision": args.precision, "cells": args.cells, "sites": H.shape[0], "moments": args.moments, "launches": nl,
                      "ms": ms, "bytes_per_launch": b, "GBps": b * nl / (ms / 1e3) / 1e9, "mu0": mu[0]}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=64)
    ap.add_argument("--fp64-moments", type=int, default=256)
    ap.add_argument("--kernel-only", action="store_true", help="small profiling case (no e2e/fp64/cpu legs)")
    ap.add_argument("--cells", type=int, default=512)
    ap.add_argument("--moments", type=int, default=32)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "dd"])
    ap.add_argument("--staged", action="store_true", help="TMA-staged warp-specialised kernel (A/B)")
    ap.add_argument("--two-step", action="store_true", help="two recursion steps per pass (A/B)")
    ap.add_argument("--kubo", type=int, default=0, choices=[0, 3, 5],
                    help="run only the Kubo leg of config 3 (sigma_xy) or 5 (sigma_xx)")
    ap.add_argument("--cuda-core-mu", action="store_true", help="Kubo leg with the CUDA-core mu GEMM")
    ap.add_argument("--kubo-recursion", default="mixed", choices=["fp64", "mixed", "dd"],
                    help="stored-block recursion: complex64 (default), double-float or complex128")
    ap.add_argument("--kubo-moments", type=int, default=0,
                    help="override M of the Kubo leg (small profiling case; not the benchmark)")
    ap.add_argument("--kubo-budget-gb", type=float, default=0.0,
                    help="stored-block budget of the Kubo leg (0: 60%% of free memory)")
    ap.add_argument("--kubo-fused", action="store_true",
                    help="Kubo leg with the output-operator products fused into the recursion (A/B)")
    ap.add_argument("--no-hopping", action="store_true",
                    help="diagonal-only H (same vector streams, no neighbour gathers): stream ceiling")
    ap.add_argument("--serve", action="store_true", help="serving stream (config 4) instead of the DoS solve")
    ap.add_argument("--serve-requests", type=int, default=4096)
    ap.add_argument("--serve-requests-default", type=int, default=512,
                    help="requests of the shortened serving stream recorded in the default line")
    ap.add_argument("--no-configs", action="store_true", help="default line without the other configurations")
    ap.add_argument("--serve-gap-ms", type=float, default=2.0)
    ap.add_argument("--serve-precision", default="mixed", choices=["mixed", "fp64", "dd"])
    ap.add_argument("--serve-budget-gb", type=float, default=120.0)
    ap.add_argument("--serve-round", type=int, default=16)
    ap.add_argument("--serve-step-gb", type=float, default=2.0)
    ap.add_argument("--serve-no-tune", action="store_true", help="serving profiling case without the tuner")
    ap.add_argument("--serve-single", action="store_true",
                    help="one honeycomb --cells^2 request through the server (profiling case)")
    ap.add_argument("--gemm", type=int, nargs=2, metavar=("M", "K"),
                    help="mu_nm GEMM alone on random M x K complex blocks (profiling case)")
    ap.add_argument("--expand", type=float, default=None, metavar="T",
                    help="time evolution exp(-iHt) of 8 vectors to time T (vector-expansion leg)")
    ap.add_argument("--small", action="store_true", help="config-1 DoS (square 64x64): latency-bound case")
    args = ap.parse_args()
    if args.small:
        print(json.dumps(run_small(args)), flush=True)
        return 0
    if args.expand is not None:
        return run_expand(args)
    if args.gemm:
        return run_gemm(args)
    if args.serve_single:
        return run_serve_single(args)
    if args.serve:
        return run_serve(args)
    if args.kernel_only:
        return run_kernel_only(args)
    if args.kubo:
        print(json.dumps(run_kubo(args.kubo, tensor=not args.cuda_core_mu, recursion=args.kubo_recursion,
                                  fuse_ops=args.kubo_fused, moments=args.kubo_moments,
                                  budget_gb=args.kubo_budget_gb)), flush=True)
        return 0
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
