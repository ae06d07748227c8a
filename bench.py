"""Benchmark: batched GMRES solves of the FFT-VIE system on one GB300.

Workload (default): ellipsoid phantom on a 128^3 grid at 2 mm, PWL basis
(12 unknowns/voxel), 297.2 MHz, 64 right-hand sides from 64 loop ports on a
16 cm cylinder; Green's tensor with the accurate near zone (the reference's
operator); block GMRES over the 64 right-hand sides (one complex64 block
Krylov space, 30 block steps per cycle, FP32 accumulation) inside an FP64
iterative-refinement loop to 1e-6 relative residual (--solver mixed: one
complex64 GMRES(50) per right-hand side instead; the line reports that
solver on the same batch beside the block one).  One step = one batched
solve of all right-hand sides, inputs resident in HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Other workloads (--workload): sphere32 (r = 6 cm sphere, 32^3 at 5 mm, PWC,
128 MHz, plane wave), ellipsoid96 (the phantom on 96^3 at 2 mm, PWL, one
loop) and uneven16 (sixteen PWC phantoms with edges 48-128 and 1-8 loops
each, the bodies on concurrent streams; reports the per-body residual
spread).  --matvec-only times operator applications alone (the small,
bounded command of the ncu captures), optionally from Tucker blocks
(--tucker pre|apply); --block-gemm M times the block solver's tensor-core
projection kernel.

Under torchrun each rank solves its own batch (replicas of the workload with
rank-seeded loop jitter; no collective on the data path), value = solves of
all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path[:0] = [str(ROOT), str(ROOT / "marie-tools_gb300")]

WORKLOADS = {
    "ellipsoid128": dict(n=128, res=2e-3, freq=297.2e6, pwl=True, nrhs=64, tol=1e-6, phantom="ellipsoid",
                 fp64_iters=183.1, tucker_ranks=(13, 13, 13),
                 desc="ellipsoid phantom 128^3 @ 2 mm, PWL, 297.2 MHz, 64 loop-port RHS"),
    "ellipsoid96": dict(n=96, res=2e-3, freq=297.2e6, pwl=True, nrhs=1, tol=1e-6, phantom="ellipsoid",
                 fp64_iters=172.0, tucker_ranks=(13, 13, 13),
                 desc="ellipsoid phantom 96^3 @ 2 mm, PWL, 297.2 MHz, 1 loop RHS"),
    "sphere32": dict(n=32, res=5e-3, freq=128e6, pwl=False, nrhs=1, tol=1e-6, phantom="sphere",
                 fp64_iters=66.0, desc="sphere r=6 cm 32^3 @ 5 mm, PWC, 128 MHz, plane wave"),
}
METRIC = "GMRES solves/s at 128^3 PWL, 1e-6 resid (mixed c64/FP64-refined, 64-RHS batch)"
BLOCK_STEPS = 30     # block Arnoldi steps per cycle of the block solver


def metric_of(wl):
    """The headline metric for the 128^3 batch; the same quantity named for
    the other workloads."""
    if wl["n"] == 128 and wl["pwl"] and wl["nrhs"] == 64:
        return METRIC
    basis = "PWL" if wl["pwl"] else "PWC"
    return (f"GMRES solves/s at {wl['n']}^3 {basis}, 1e-6 resid (mixed c64/FP64-refined, "
            f"{wl['nrhs']}-RHS batch)")


# tucker_ranks: ranks of the Tucker blocks the reference re-expands in every
# product (its CPU arm); the mean HOSVD ranks at the reference's tolerance
# 1e-7 (load_inputs.m:69) of the PWL N operator at 2 mm / 297.2 MHz measured
# on 24^3 (12.0) and 48^3 (13.2) grids, rounded down (larger grids have
# larger ranks, so the reference arm is not made slower than it is).
# fp64_iters (per workload above): FP64 GMRES(50) iterations per right-hand
# side to 1e-6 on the workload's own operator (Green's tensor with the
# accurate near zone), measured by this library's complex128 solver, which
# follows is_gmres_vie.m / is_iter_gmres_vie.m step for step and matches
# the oracle's iteration counts on every case the tests compare: 128^3, the
# mean over the first 16 loop ports (171-190); 96^3, the one loop; 32^3, the
# plane wave (two restart cycles).  Our arm re-measures them in every run
# ('fp64_gpu.iters_mean'); the reference arm, which runs the CPU port of the
# reference's algorithm and cannot afford a full 128^3 FP64 solve on the
# host, turns its per-iteration time into solves/s with them.


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def build_problem(wl, rank, torch):
    """Phantom, GPU-assembled operator and right-hand sides of one workload."""
    from marie_gb300 import VieOperator, assemble_green, phantoms
    n, res, freq, pwl = wl["n"], wl["res"], wl["freq"], wl["pwl"]
    if wl["phantom"] == "sphere":
        body = phantoms.sphere(n, res, 0.06, 50.0, 0.6)
    else:
        body = phantoms.ellipsoid_phantom(n, res, seed=0)
    emc = phantoms.em_constants(freq)
    t0 = time.time()
    ivN = assemble_green(body.n, res, freq, pwl, "N", near=wl.get("near", "relative"))
    t_asm = time.time() - t0
    # complex64 inner solves + complex128 (float-float arithmetic) residuals
    op = VieOperator(body.n, res, freq, body.idx_solution(pwl), body.Mr(freq), ivN, pwl=pwl,
                     precisions=(2 | 4) if n % 16 == 0 and n <= 128 else 3, max_rhs=wl["nrhs"])
    del ivN
    if wl["phantom"] == "sphere":
        Ue = op.incident_plane_wave(body.origin).reshape(1, -1).repeat(wl["nrhs"], 1)
    elif wl["nrhs"] == 1:
        loops, radius = phantoms.loop_outside((0.080, 0.065, 0.090), gap=0.01, radius=0.05)
        Ue = op.incident_loops(body.origin, loops, radius, nseg=64).reshape(1, -1)
    else:
        loops = phantoms.loop_ring(wl["nrhs"], ring_radius=0.16, seed=1 + rank)
        Ue = op.incident_loops(body.origin, loops, 0.025, nseg=64).reshape(wl["nrhs"], -1)
    Mr = body.Mr(freq).reshape(-1, order="F")[body.idxS]
    chi = np.tile((1.0 / Mr) * (Mr - 1.0), 12 if pwl else 3)
    b = (emc["ce"] * torch.from_numpy(chi).cuda()[None, :] * Ue).contiguous()   # ie_solver_vie.m:18
    return op, body, b.reshape(-1), t_asm


def solve_alg_bytes(n, pwl, Nb, iters, n_c128, chunk, restart=50, block_steps=0, cycles=None):
    """Algorithmic bytes of one batched mixed solve by the fixed per-matvec
    and per-Arnoldi-step formulas: per right-hand side, `iters[r]` complex64
    matvecs of 26 n^3 C s bytes plus the Green spectrum U (n+1)^3 s shared by
    the `chunk` right-hand sides of a launch, and `n_c128` complex128
    true-residual matvecs (s = 16).  Per-RHS GMRES: Arnoldi step k of a cycle
    (2k + 4) N_b s bytes.  Block GMRES (block_steps > 0, `cycles[r]` cycles):
    block step j reads V_{0:j} twice (projection, update; (j+1) vectors per
    right-hand side each) and W six times (update, two Gram matrices, two
    normalisations, the copy) and writes it four times: (2(j+1) + 10) N_b s
    per right-hand side."""
    C, U = (12, 60) if pwl else (3, 6)

    def mv(s):
        return 26 * n ** 3 * C * s + U * (n + 1) ** 3 * s / chunk

    total = 0.0
    its = np.asarray(iters, dtype=np.int64).reshape(-1)
    for r, it in enumerate(its):
        it = int(it)
        if block_steps > 0:
            ncyc = max(1, int(cycles[r]))
            per = it / ncyc           # steps of a cycle (the cycles' mean)
            steps = ncyc * sum(2 * (j + 1) + 10 for j in range(int(round(per))))
        else:
            full, rem = divmod(it, restart)
            steps = full * (restart * (restart + 1) + 4 * restart) + rem * (rem + 1) + 4 * rem   # sum of (2k + 4)
        total += it * mv(8) + steps * Nb * 8 + n_c128 * mv(16)
    return total


def roofline_z(op, wl, tiles, ms_z, peak, peak_kind, zfrac=1.0):
    """Algorithmic bytes of one z-pass launch / its event-timed duration.
    zfrac: fraction of z slices holding body voxels (the pass reads and
    writes those only)."""
    n, C = wl["n"], 12 if wl["pwl"] else 3
    U = 60 if wl["pwl"] else 6
    s = 8                                   # complex64
    units = min(tiles["chunk"], wl["nrhs"])  # right-hand sides per launch
    per_rhs = 8 * n ** 3 * C * s * zfrac    # read + write 4 n^3 per component (live slices)
    green = U * (n + 1) ** 3 * s            # octant spectrum, read once per launch
    alg = units * per_rhs + green
    achieved = alg / (ms_z * 1e-3) / 1e9
    # DRAM traffic of the launch: the ncu capture of k4_zp<6,PWL> on the 96^3
    # ellipsoid with 4 right-hand sides (read + write bytes per launch, one
    # kernel, `--metrics dram__bytes_read.sum,dram__bytes_write.sum`) set
    # against the byte model of that launch (live slices read and written
    # once, the full Green spectrum read once), and the same ratio applied to
    # this launch's model.  A capture at this workload's size would hold tens
    # of GB on the device.
    traffic = None
    if wl["pwl"] and n % 16 == 0 and 16 <= n <= 128:
        full = U * (2 * n) ** 3 * s                                     # full spectrum, pair layout
        model = units * per_rhs + full
        model96 = 4 * 8 * 96 ** 3 * 12 * 8 * Z96_LIVE + 60 * 192 ** 3 * 8
        traffic = int(model * (Z96_DRAM_BYTES / model96))
    four_step = n % 16 == 0 and 16 <= n <= 128
    name = (f"k4_zp<{n // 16},{'PWL' if wl['pwl'] else 'PWC'}>" if four_step else "k_z<float>")
    # FP32 work of the same launch: per right-hand side and (kx, ky) column,
    # C forward + C inverse zero-padded transforms (two n-point halves each,
    # 5 m log2 m flops per m-point transform, plus 6 flops per point for the
    # odd half's w_2n twist) and the Green product (C*C complex multiply-adds,
    # 8 flops each, at 2n frequencies); against the FP32 FMA rate of 152 SMs
    # x 128 lanes x 2 flops at the SM clock sampled during the run
    fft = 2 * C * (2 * 5 * n * math.log2(n) + 6 * n)
    prod = 2 * n * C * C * 8
    flops = units * (2 * n) ** 2 * (fft + prod)
    return {"kernel": name + " (z FFT + Green block multiply + inverse z FFT)", "bound": "hbm",
            "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "traffic": traffic, "alg_bytes_per_launch": int(alg), "launch_ms": round(ms_z, 4),
            "traffic_source": ("ncu DRAM read+write of the same kernel on the 96^3 ellipsoid with 4 right-hand "
                               "sides, scaled to this launch by its byte model (live slices once, full Green "
                               "spectrum once)") if traffic else None,
            "units_per_launch": units, "peak_source": peak_kind,
            "fp32": {"flops_per_launch": int(flops), "achieved_tflops": round(flops / (ms_z * 1e-3) / 1e12, 2)}}


# ncu, k4_zp<6,PWL> on the 96^3 ellipsoid (4 right-hand sides, live slice
# fraction 0.9375): dram__bytes_read.sum + dram__bytes_write.sum per launch
Z96_DRAM_BYTES = 4671918080 + 1248136960
Z96_LIVE = 0.9375


def run_ours(args, wl):
    import torch
    import torch.distributed as dist
    from marie_gb300 import _lib
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as ge
    if rank == 0:
        ge.build()
    if ws > 1:
        dist.barrier()
    ge.build()
    op, body, b, t_asm = build_problem(wl, rank, torch)
    nrhs = wl["nrhs"]
    # the right-hand sides of a batch share one block Krylov space (block
    # GMRES, 30 block steps per cycle); one right-hand side runs the
    # per-RHS mixed solver
    solver = args.solver or ("block" if nrhs >= 8 else "mixed")
    kw = dict(restart=50, tol=wl["tol"], maxit=200, mode=solver, inner_tol=1e-7, block_steps=BLOCK_STEPS)
    # warm-up (also the solve whose statistics are reported)
    rep = None
    for _ in range(args.warmup):
        x, rep = op.gmres(b, **kw)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    launches0 = _lib.launch_count()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            x, rep = op.gmres(b, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = _lib.launch_count() - launches0
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if ws > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = nrhs * args.steps * ws / (ms_max * 1e-3)

    # end to end through the public API on host buffers (marie_gmres_vie_host:
    # pinned b in, x out, copies inside the timed region; the per-RHS solver
    # overlaps them with its chunks, the block solver takes the whole batch
    # as one block)
    b_host = b.cpu().pin_memory()
    x_host = torch.empty_like(b_host).pin_memory()
    # warm-up of the host path's own device buffers: a loose tolerance ends
    # each chunk after one iteration (the solver workspace is already sized)
    op.gmres_host(b_host, out=x_host, **dict(kw, tol=0.5, maxit=1))
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e2.record(stream)
    nE = 1
    for _ in range(nE):
        op.gmres_host(b_host, out=x_host, **kw)
    e3.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e2.elapsed_time(e3) / nE
    e2e = {"value": round(nrhs * ws / (ms_e2e * 1e-3), 4), "unit": "solves/s",
           "h2d_bytes_per_step": int(b_host.numel() * 16), "d2h_bytes_per_step": int(x_host.numel() * 16)}

    # roofline of the dominant kernel (z pass, complex64) with CUDA events
    peak, peak_kind = measured_peaks()
    tiles = op.tiles()
    xs = b[: op.Nb * min(nrhs, tiles["chunk"])].to(torch.complex64)
    passes = op.profile(xs, reps=5)
    zlive = np.unique(body.idxS // (body.n[0] * body.n[1])).size / body.n[2]
    roof = roofline_z(op, wl, tiles, passes[2], peak, peak_kind, zfrac=zlive)
    roof["live_z_fraction"] = round(float(zlive), 4)
    n, C, s = wl["n"], 12 if wl["pwl"] else 3, 8
    U = 60 if wl["pwl"] else 6
    units = xs.numel() // op.Nb
    bmv = 26 * n ** 3 * C * s * units + U * (n + 1) ** 3 * s
    roof["matvec"] = {"ms": round(passes[5], 4), "rhs": units, "alg_bytes": bmv,
                      "achieved_GBs": round(bmv / (passes[5] * 1e-3) / 1e9, 1),
                      "pass_ms": [round(v, 4) for v in passes[:5]]}

    # The plain complex128 GMRES (the drop-in for is_gmres_vie) against the
    # mixed solver, like for like: both batched over the same first
    # right-hand sides (one matvec chunk), each timed with CUDA events on the
    # same operator.  Right-hand sides are solved in chunks one after another
    # inside a call, so solves/s of one chunk is that of the whole batch.
    fp64 = None
    if not args.skip_fp64:
        nb = min(nrhs, tiles["chunk"])
        bb = b[: nb * op.Nb].clone()
        f0, f1, f2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        f0.record(stream)
        xm, repm = op.gmres(bb, **kw)
        f1.record(stream)
        x64, rep64 = op.gmres(bb, restart=50, tol=wl["tol"], maxit=200, mode="fp64")
        f2.record(stream)
        torch.cuda.synchronize()
        ms_m, ms_64 = f0.elapsed_time(f1), f1.elapsed_time(f2)
        X32, X64 = xm.reshape(nb, op.Nb), x64.reshape(nb, op.Nb)
        ferr = (torch.linalg.norm(X32 - X64, dim=1) / torch.linalg.norm(X64, dim=1)).cpu().numpy()
        fp64 = {"operator": "complex128, float-float arithmetic" if op.tiles(0)["float_float"] else "complex128, FP64",
                "batch_rhs": nb, "solves_per_s": round(nb / (ms_64 * 1e-3), 5),
                "iters_mean": float(np.mean(rep64.iters)), "iters_min_max": [int(rep64.iters.min()), int(rep64.iters.max())],
                "true_resid_max": float(rep64.true_resid.max()), "converged": int(np.sum(rep64.status == 0)),
                "mixed_same_batch_solves_per_s": round(nb / (ms_m * 1e-3), 5),
                "mixed_over_fp64": round(ms_64 / ms_m, 3),
                "field_err_mixed_vs_fp64_max": float(ferr.max())}

    # the per-right-hand-side mixed solver on the same batch, for comparison
    per_rhs = None
    if solver == "block" and not args.skip_fp64:
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        g0.record(stream)
        xp, repp = op.gmres(b, **dict(kw, mode="mixed"))
        g1.record(stream)
        torch.cuda.synchronize()
        ms_p = g0.elapsed_time(g1)
        XB, XP = x.reshape(nrhs, op.Nb), xp.reshape(nrhs, op.Nb)
        dif = (torch.linalg.norm(XB - XP, dim=1) / torch.linalg.norm(XP, dim=1)).cpu().numpy()
        per_rhs = {"solver": "complex64 GMRES(50) per right-hand side + FP64 refinement", "batch_rhs": nrhs,
                   "solves_per_s": round(nrhs / (ms_p * 1e-3), 4), "iters_mean": float(np.mean(repp.iters)),
                   "matvecs_c64": int(repp.matvecs_c64), "true_resid_max": float(repp.true_resid.max()),
                   "block_over_per_rhs": round(ms_p / (ms_max / args.steps), 3),
                   "solution_diff_max": float(dif.max())}

    cpu = None
    if rank == 0 and not args.skip_cpu:
        cpu = cpu_baseline(wl, iters=(fp64["iters_mean"] if fp64 else wl["fp64_iters"]), budget_s=args.cpu_budget)
    clocks = clk.summary()
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if sm_mhz:
        nsm = torch.cuda.get_device_properties(local).multi_processor_count
        fp32_peak = nsm * 128 * 2 * sm_mhz * 1e6 / 1e12
        roof["fp32"].update({"peak_tflops": round(fp32_peak, 2), "frac": round(roof["fp32"]["achieved_tflops"] / fp32_peak, 4),
                             "peak_source": f"nominal: {nsm} SMs x 128 FP32 lanes x 2 flops x {sm_mhz:.0f} MHz (sampled)"})
    # whole-solve bytes by the fixed formulas over the measured step time
    try:
        alg = solve_alg_bytes(wl["n"], wl["pwl"], op.Nb, rep.iters, int(rep.matvecs_c128),
                              min(nrhs, tiles["chunk"]), block_steps=BLOCK_STEPS if solver == "block" else 0,
                              cycles=rep.outer)
        solve_roofline = {"bound": "hbm", "alg_bytes_per_step": int(alg),
                          "achieved": round(alg / (ms_max / args.steps * 1e-3) / 1e9, 1), "unit": "GB/s",
                          "peak": peak, "frac": round(alg / (ms_max / args.steps * 1e-3) / 1e9 / peak, 4),
                          "peak_source": peak_kind,
                          "model": "per RHS: iters x c64 matvec (26 n^3 C 8 B + Green/chunk) + Arnoldi bytes "
                                   "(per-RHS: sum_k (2k+4) N_b 8 B; block: sum_j (2(j+1)+10) N_b 8 B) "
                                   "+ c128 residual matvecs (16 B)"}
    except Exception as e:      # a reported extra: never fail the run over it
        solve_roofline = {"error": repr(e)}
    if rank == 0:
        line = {
            "metric": metric_of(wl), "value": round(value, 4), "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 (FP32 accumulation) + FP64 refinement",
            "data": "synthetic (seeded phantom, GPU-assembled Green's tensor, loop incident fields)",
            "config": {"workload": wl["desc"], "grid": [wl["n"]] * 3, "basis": "PWL" if wl["pwl"] else "PWC",
                       "near_zone": wl.get("near", "relative"),
                       "n_body_voxels": int(body.idxS.size), "unknowns_per_rhs": int(op.Nb),
                       "rhs_per_gpu": nrhs, "tol": wl["tol"],
                       "solver": (f"block GMRES, {BLOCK_STEPS} block steps per cycle, one block of {nrhs} RHS, "
                                  "FP64 refinement" if solver == "block" else
                                  "complex64 GMRES(50) per RHS, FP64 refinement"),
                       "l2": "inputs larger than L2 (Krylov basis and FFT work arrays are tens of GB)",
                       "parallelism": f"replicas x{ws} (independent RHS batches, no collective)"},
            "e2e": e2e, "gpu_launches": int(launches),
            "clocks": clocks, "roofline": roof, "cpu_baseline": cpu,
            "solve": {"iters_per_rhs_mean": float(np.mean(rep.iters)), "matvecs_c64": int(rep.matvecs_c64),
                      "matvecs_c128": int(rep.matvecs_c128), "true_resid_max": float(np.max(rep.true_resid)),
                      "converged": int(np.sum(rep.status == 0))},
            "fp64_gpu": fp64, "per_rhs_mixed": per_rhs, "assembly_s": round(t_asm, 2),
            "solve_roofline": solve_roofline,
        }
        print(json.dumps(line), flush=True)
    op.close()
    if ws > 1:
        dist.destroy_process_group()


def cpu_baseline(wl, iters, budget_s=30.0, steps=1, warmup=0, tucker_ranks=None):
    """Time the CPU oracle (FP64 numpy/scipy restatement of mvp_vie + one
    classical Gram-Schmidt Arnoldi step) on the full-size workload, all host
    cores, and convert to solves/s with `iters` GMRES iterations per solve.
    tucker_ranks: re-expand Tucker blocks of these ranks inside every block
    product, as the reference does (mvp_N_pwl_tucker.m:31); None: Green
    blocks pre-expanded."""
    from oracle import cpu_bench
    r = cpu_bench.time_iteration(wl["n"], wl["pwl"], steps=steps, warmup=warmup, budget_s=budget_s,
                                 tucker_ranks=tucker_ranks)
    sec_iter = r["sec_per_iter"]
    blocks = (f"Tucker blocks of ranks {tuple(tucker_ranks)} re-expanded in every product" if tucker_ranks
              else "pre-expanded Green blocks")
    return {"value": round(1.0 / (sec_iter * iters), 6), "unit": "solves/s", "cores": r["cores"], "kind": "port",
            "sample": (f"{r['iters_timed']} GMRES iteration(s) (one FP64 mvp_vie with {blocks} + "
                       f"one CGS Arnoldi step at k={r['k']}) on the full {wl['n']}^3 grid, "
                       f"{r['sec_per_iter']:.2f} s each, x {iters} iterations/solve"),
            "sec_per_iter": round(sec_iter, 3)}


def run_reference(args, wl):
    ws, rank, local = _dist()
    if rank != 0:
        return
    # the reference's own form of the algorithm: Tucker blocks re-expanded in
    # every product (PWL workloads; PWC has 9 expansions per matvec, timed
    # pre-expanded); the pre-expanded form is timed beside it for reference
    ranks = wl.get("tucker_ranks")
    cpu = cpu_baseline(wl, iters=wl["fp64_iters"], budget_s=1e9, steps=args.steps, warmup=args.warmup,
                       tucker_ranks=ranks)
    pre = cpu_baseline(wl, iters=wl["fp64_iters"], budget_s=60.0, steps=max(1, args.steps), warmup=0) if ranks \
        else None
    line = {"impl": "reference", "metric": metric_of(wl), "value": cpu["value"], "unit": "solves/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": wl["desc"], "grid": [wl["n"]] * 3, "rhs_per_gpu": wl["nrhs"],
                       "note": "MATLAB reference cannot run here; its FP64 algorithm (mvp_vie with the Tucker "
                               "blocks re-expanded in every product for PWL, mvp_N_pwl_tucker.m:31; single-pass CGS "
                               "Arnoldi) is timed as the numpy/scipy port on the host cores; cpu_pre_expanded times "
                               "the same with the blocks expanded once"},
            "cpu_baseline": cpu, "cpu_pre_expanded": pre,
            "e2e": {"value": cpu["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_matvec_only(args, wl):
    """Operator applications only (no solver state on the device): the small,
    bounded command used for ncu captures of the matvec kernels."""
    import torch
    import __graft_entry__ as ge
    from marie_gb300 import VieOperator, assemble_green, phantoms
    ge.build()
    torch.cuda.set_device(0)
    n, res, freq, pwl = wl["n"], wl["res"], wl["freq"], wl["pwl"]
    body = phantoms.ellipsoid_phantom(n, res, seed=0) if wl["phantom"] != "sphere" else phantoms.sphere(n, res)
    ivN = assemble_green(body.n, res, freq, pwl, "N", near=wl.get("near", "relative"))
    prec = {"c64": 2, "c128": 1, "c128ff": 4}[args.prec]
    extra = {}
    if args.tucker != "none":
        # the reference's operator format: blocks compressed at its tolerance 1e-7
        from marie_gb300 import tucker
        t0 = time.time()
        ivN = tucker.compress(ivN, 1e-7)
        r = tucker.ranks(ivN)
        extra = {"tucker": args.tucker, "ranks_mean": float(r.mean()), "ranks_max": int(r.max()),
                 "compress_s": round(time.time() - t0, 1)}
        if args.tucker == "apply":
            prec |= 8
    op = VieOperator(body.n, res, freq, body.idx_solution(pwl), body.Mr(freq), ivN, pwl=pwl, precisions=prec,
                     max_rhs=wl["nrhs"])
    del ivN
    dt = torch.complex64 if args.prec == "c64" else torch.complex128
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(wl["nrhs"] * op.Nb, dtype=dt, device="cuda", generator=g)
    for _ in range(args.matvec_only):
        op.apply(x)
    torch.cuda.synchronize()
    ms = op.profile(x, reps=3)
    # whole applications (the per-application Tucker expansion runs ahead of the passes)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        op.apply(x)
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"matvec_only": wl["desc"], "prec": args.prec, "nrhs": wl["nrhs"],
                      "pass_ms": [round(v, 4) for v in ms[:5]], "matvec_ms": round(ms[5], 4),
                      "apply_ms": round(e0.elapsed_time(e1) / 3, 4), **extra}), flush=True)
    op.close()


def run_block_gemm(args):
    """The block solver's tensor-core projection H = V^H W (marie_block_gemm_cn)
    on seeded complex64 data of the solver's shape: N_b rows, M basis
    vectors, 64 right-hand sides; CUDA-event time over 5 calls after 3, bytes
    read (V once, W once per 512-column tile) and the error against a
    complex128 product (per entry, relative to ||V_a|| ||W_c||)."""
    import ctypes as ct
    import torch
    import __graft_entry__ as ge
    from marie_gb300 import _lib
    ge.build()
    lib = _lib.load()
    K, M, p = args.block_gemm_rows, args.block_gemm, 64
    g = torch.Generator(device="cuda").manual_seed(0)
    V = torch.randn(M * K, dtype=torch.complex64, device="cuda", generator=g)
    W = torch.randn(p * K, dtype=torch.complex64, device="cuda", generator=g)
    H = torch.zeros(M * p, dtype=torch.complex64, device="cuda")
    nf = lib.marie_block_gemm_part_floats(K, M)
    part = torch.empty(nf, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call():
        st = lib.marie_block_gemm_cn(ct.c_void_p(V.data_ptr()), K, ct.c_void_p(W.data_ptr()), K, K, M, p,
                                     ct.c_void_p(H.data_ptr()), M, ct.c_void_p(part.data_ptr()), nf,
                                     ct.c_void_p(err.data_ptr()), stream)
        _lib.check(st)

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        call()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 5
    Vm, Wm = V.reshape(M, K), W.reshape(p, K)
    ref = torch.zeros(M, p, dtype=torch.complex128, device="cuda")
    for k0 in range(0, K, 1 << 18):
        ref += Vm[:, k0:k0 + (1 << 18)].to(torch.complex128).conj() @ Wm[:, k0:k0 + (1 << 18)].to(torch.complex128).T
    bound = (torch.linalg.norm(Vm.to(torch.complex128), dim=1)[:, None] *
             torch.linalg.norm(Wm.to(torch.complex128), dim=1)[None, :])
    rel = ((H.reshape(p, M).T.to(torch.complex128) - ref).abs() / bound).max().item()
    nbytes = (M + p * ((M + 511) // 512)) * K * 8
    print(json.dumps({"block_gemm": {"rows": K, "basis_vectors": M, "rhs": p}, "ms": round(ms, 4),
                      "bytes": nbytes, "achieved_GBs": round(nbytes / (ms * 1e-3) / 1e9, 1),
                      "rel_err_max": rel, "wait_expired": int(err.item())}), flush=True)


def uneven_instances(seed=44, count=16, res=2e-3):
    """The uneven-size batch: `count` seeded PWC phantoms with grid edges drawn
    from {48, ..., 128} at 2 mm, 128 or 297.2 MHz, 1-8 loops on a ring around
    each body, bodies scaled to their grid (the same generator as the
    sixteen-phantom parity test)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.choice([48, 64, 80, 96, 112, 128]))
        freq = float(rng.choice([128e6, 297.2e6]))
        nl = int(rng.integers(1, 9))
        out.append(dict(i=i, n=n, freq=freq, nloops=nl, res=res, scale=0.9 * (n * res / 2) / 0.090))
    return out


def _concurrent(torch, insts, fn, nstreams):
    """Run fn(inst) for every instance, the instances dealt round-robin to
    `nstreams` host threads, each on its own CUDA stream (the library's GMRES
    host loop synchronises only its own stream, so the bodies' kernels
    overlap on the GPU).  Returns after every stream is done."""
    import threading
    groups = [insts[i::nstreams] for i in range(nstreams)]
    streams = [torch.cuda.Stream() for _ in groups]
    start = torch.cuda.Event()
    start.record(torch.cuda.current_stream())
    errors = []

    def work(g, st):
        try:
            with torch.cuda.stream(st):
                st.wait_event(start)
                for inst in g:
                    fn(inst)
        except Exception as e:      # surfaced after the join
            errors.append(e)

    th = [threading.Thread(target=work, args=(g, st)) for g, st in zip(groups, streams)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for st in streams:
        torch.cuda.current_stream().wait_stream(st)
    if errors:
        raise errors[0]


def run_uneven(args):
    """Sixteen independent PWC bodies of uneven grid size, every loop of every
    body solved to 1e-6 (mixed complex64 / FP64-refined GMRES) per step, each
    body as one batched solve of its loops.  The bodies run concurrently on
    `--streams` CUDA streams (host threads); each body's z-pass tile was
    picked by the library's autotuner at set-up.  value = loops solved /
    time; per-instance iterations and true residuals give the spread."""
    import torch
    import __graft_entry__ as ge
    from marie_gb300 import VieOperator, assemble_green, phantoms, _lib
    ge.build()
    torch.cuda.set_device(0)
    t0 = time.time()
    insts = []
    tuned = []
    for d in uneven_instances():
        n, res, freq, nl = d["n"], d["res"], d["freq"], d["nloops"]
        body = phantoms.ellipsoid_phantom(n, res, seed=100 + d["i"], scale=d["scale"])
        iv = assemble_green(body.n, res, freq, False, "N", near=args.near)
        op = VieOperator(body.n, res, freq, body.idx_solution(False), body.Mr(freq), iv, pwl=False,
                         precisions=2 | 4, max_rhs=nl)
        del iv
        loops = phantoms.loop_ring(nl, ring_radius=0.080 * d["scale"] + 0.01, z_extent=0.0, n_angles=nl,
                                   seed=200 + d["i"])
        Ue = op.incident_loops(body.origin, loops, 0.25 * n * res / 2, nseg=64).reshape(nl, -1)
        ce = phantoms.em_constants(freq)["ce"]
        Mr = body.Mr(freq).reshape(-1, order="F")[body.idxS]
        chi = np.tile((1.0 / Mr) * (Mr - 1.0), 3)
        b = (ce * torch.from_numpy(chi).cuda()[None, :] * Ue).reshape(-1).contiguous()
        t = op.autotune(b.to(torch.complex64), reps=3)
        tuned.append({"grid": n, "loops": nl, "z_tile_ms": {str(k): round(v, 4) for k, v in t.items()},
                      "chosen": op.tiles()["width"]})
        insts.append((d, op, b))
    t_setup = time.time() - t0
    kw = dict(restart=50, tol=1e-6, maxit=200, mode="mixed", inner_tol=1e-7, block_steps=BLOCK_STEPS)
    reps = {}

    def mode_of(op, b):
        # per-RHS mixed by default: the block solver's host synchronisations
        # per block step (block QR, least squares) cost more than its fewer
        # operator applications save on these small bodies (block GMRES for
        # the multi-loop bodies: 12.5 against 18.0 solves/s on four streams)
        return args.solver or "mixed"

    def solve(inst):
        d, op, b = inst
        reps[d["i"]] = op.gmres(b, **dict(kw, mode=mode_of(op, b)))[1]

    for _ in range(max(1, args.warmup)):
        _concurrent(torch, insts, solve, args.streams)
    torch.cuda.synchronize()
    launches0 = _lib.launch_count()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            _concurrent(torch, insts, solve, args.streams)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = _lib.launch_count() - launches0
    total = sum(d["nloops"] for d, _, _ in insts)
    # end to end: host right-hand sides in, host solutions out, per body
    hb = [(op, b.cpu().pin_memory()) for _, op, b in insts]
    hx = [torch.empty_like(b).pin_memory() for _, b in hb]
    hio = list(zip(hb, hx))

    def solve_host(item):
        (op, b), x = item
        op.gmres_host(b, out=x, **dict(kw, mode=mode_of(op, b)))

    _concurrent(torch, hio, solve_host, args.streams)
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e2.record(stream)
    _concurrent(torch, hio, solve_host, args.streams)
    e3.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e2.elapsed_time(e3)
    per = []
    for d, op, _ in insts:
        r = reps[d["i"]]
        per.append({"grid": d["n"], "freq_MHz": d["freq"] / 1e6, "loops": d["nloops"], "unknowns": int(op.Nb),
                    "iters_mean": round(float(np.mean(r.iters)), 2), "true_resid_max": float(np.max(r.true_resid)),
                    "converged": int(np.sum(r.status == 0))})
    tr = np.array([p["true_resid_max"] for p in per])
    line = {
        "metric": "GMRES solves/s, uneven-size batch of 16 PWC phantoms (edges 48-128, 1-8 loops each), 1e-6 resid",
        "value": round(total * args.steps / (ms * 1e-3), 4), "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 (FP32 accumulation) + FP64 refinement",
        "data": "synthetic (seeded phantoms, GPU-assembled Green's tensors, loop incident fields)",
        "config": {"workload": "16 PWC ellipsoid phantoms, edges from {48..128} at 2 mm, 128/297.2 MHz, 1-8 loops",
                   "loops_total": total, "restart": 50, "tol": 1e-6, "near_zone": args.near,
                   "schedule": f"bodies on {args.streams} concurrent CUDA streams (host threads), each body one "
                               "batched solve of its loops; z-pass tiles from the library's autotuner",
                   "solver": args.solver or "mixed"},
        "e2e": {"value": round(total / (ms_e2e * 1e-3), 4), "unit": "solves/s",
                "h2d_bytes_per_step": int(sum(b.numel() * 16 for _, b in hb)),
                "d2h_bytes_per_step": int(sum(x.numel() * 16 for x in hx))},
        "gpu_launches": int(launches), "clocks": clk.summary(),
        "residual_spread": {"min": float(tr.min()), "median": float(np.median(tr)), "max": float(tr.max())},
        "instances": per, "setup_s": round(t_setup, 2), "autotune": tuned,
    }
    print(json.dumps(line), flush=True)
    for _, op, _ in insts:
        op.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ellipsoid128", choices=sorted(WORKLOADS) + ["uneven16"])
    ap.add_argument("--nrhs", type=int, default=None)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=30.0)
    ap.add_argument("--streams", type=int, default=4, help="uneven16: concurrent CUDA streams for the bodies")
    ap.add_argument("--block-gemm", type=int, default=0, metavar="M",
                    help="profiling aid: the block solver's tensor-core projection V^H W (M basis vectors, "
                         "--block-gemm-rows rows, 64 right-hand sides) on seeded data, timed")
    ap.add_argument("--block-gemm-rows", type=int, default=2939712)
    ap.add_argument("--matvec-only", type=int, default=0,
                    help="profiling aid: build the workload, apply mvp_vie this many times, print per-pass times")
    ap.add_argument("--near", default="relative", choices=["standin", "relative"],
                    help="near zone of the assembled Green's tensor: the accurate host cubature that matches the "
                         "reference's surface-surface near zone (default), or the staggered GPU stand-in cubature")
    ap.add_argument("--tucker", default="none", choices=["none", "pre", "apply"],
                    help="--matvec-only: build the operator from Tucker blocks (tolerance 1e-7) expanded once at "
                         "create (pre) or re-expanded in every complex64 application (apply)")
    ap.add_argument("--solver", default=None, choices=["block", "mixed"],
                    help="inner solver (default: block for batches of 8 or more right-hand sides)")
    ap.add_argument("--prec", default="c64", choices=["c64", "c128", "c128ff"],
                    help="precision of --matvec-only (c128ff: complex128 in float-float arithmetic)")
    args = ap.parse_args()
    if args.workload == "uneven16":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the uneven-size batch is timed for this "
                              "library only; the reference arm times the 128^3 PWL workload"}), flush=True)
        elif _dist()[1] == 0:
            run_uneven(args)
        return
    wl = dict(WORKLOADS[args.workload])
    wl["near"] = args.near
    if args.nrhs:
        wl["nrhs"] = args.nrhs
    if args.block_gemm:
        run_block_gemm(args)
        return
    if args.matvec_only:
        run_matvec_only(args, wl)
        return
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()
