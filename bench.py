"""Benchmark of the explicit residual-and-update path on one GB300.

Workload (headline): Mach-2 shock hitting a density-3 sphere on a 128^3
hexahedral mesh handled as unstructured faces/cells (2,097,152 cells,
6.24M interior faces), HLLC flux, second-order LSQ reconstruction with the
Barth-Jespersen limiter (frame-invariant velocity limiting), Wray 3-stage RK,
CFL 0.4.  A "step" is one time step: the CFL time-step reduction plus three
RK stages on the device.

  value  Mcell*RK-stage/s of the mixed FP32/FP64 path, state resident in HBM
  fp64   the same metric for the all-FP64 path, and the mixed-vs-FP64
         L1/Linf density and pressure differences after the configured 500
         steps from the same initial state (and after 100 and 250)
  e2e    Mcell*RK-stage/s through the C ABI with host buffers: every step
         uploads cv from pinned host memory, steps, and downloads cv
  roofline  dominant kernel of the mixed path against the measured HBM copy
         bandwidth
  tets   the same metric on the 64^3 x 6 jittered-tetrahedron blast mesh
         (1,572,864 cells), HLLC + Barth-Jespersen, mixed and FP64, with
         its whole-stage roofline at the mesh's measured S and Nf/Nc
  cpu_baseline  the CPU oracle (the FP64 restatement of the reference,
         OpenMP over all host cores) on a bounded sample of the same 128^3
         workload: a few whole steps, plus one step on one thread
  weno   the same workload with WENO-XYZ smoothing + the simple limiter
         (RECONST 2, the solver's default), mixed and FP64
  adjoint, unrolled_adjoint  VJP/primal cost and central-difference checks
         of the residual's adjoint (tetrahedral case; componentwise BJ, the
         eigen-frame BJ and WENO-XYZ) and of the checkpointed time-unrolled
         adjoint (64^3 blast)

The working set (state, gradients, face fluxes, geometry: > 0.5 GB) is far
larger than the 126 MB L2, so no L2 flush is needed between steps.

--impl reference times the CPU restatement of the reference path on the same
128^3 workload with all host cores (OpenMP; per cell the same sums in the
reference's order, so results do not depend on the thread count), one whole
time step per bench step; the Fortran reference cannot be built here.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Mcell*RK-stage/s (mixed FP32/FP64 path; FP64 path and L1 rho error reported beside it)"
UNIT = "Mcell*RK-stage/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=128, help="cells per side of the hex box")
    p.add_argument("--cpu-steps", type=int, default=3, help="whole steps of the all-core CPU sample")
    p.add_argument("--accuracy-steps", type=int, default=500, help="steps of the mixed-vs-FP64 comparison")
    p.add_argument("--skip-tets", action="store_true", help="skip the tetrahedral-mesh throughput block")
    p.add_argument("--tet-n", type=int, default=64, help="hexes per side of the tet blast mesh (x6 tets)")
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--skip-e2e", action="store_true")
    p.add_argument("--precisions", default="mixed,fp64", help="device paths to time (profiling runs time one)")
    p.add_argument("--skip-adjoint", action="store_true")
    p.add_argument("--adj-n", type=int, default=32, help="hexes per side of the tet adjoint case")
    p.add_argument("--only-adjoint", action="store_true", help="time the adjoint case only")
    p.add_argument("--adj-reconst", type=int, default=100,
                   help="RECONST of --only-adjoint (100 componentwise BJ, 10 eigen-frame BJ, 2 WENO-XYZ, ...)")
    p.add_argument("--skip-unrolled", action="store_true", help="skip the time-unrolled adjoint case")
    p.add_argument("--skip-weno", action="store_true", help="skip the WENO-XYZ (RECONST 2) variant")
    p.add_argument("--unrolled-n", type=int, default=64, help="hexes per side of the unrolled-adjoint blast")
    p.add_argument("--unrolled-steps", type=int, default=200)
    p.add_argument("--unrolled-every", type=int, default=20, help="checkpoint interval (steps)")
    p.add_argument("--unrolled-fd", type=int, default=16, help="finite-difference directions")
    return p.parse_args()


def max_over_ranks(x, device=None):
    """The maximum of x over the ranks of the default process group (x itself
    when the job is not distributed): the slowest rank's time."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(units_per_rank, world_size, ms):
    """Mcell*RK-stage/s of the whole job: the cell-stages all ranks processed
    (each rank runs its own region: replicas) over the slowest rank's ms."""
    return world_size * units_per_rank / (ms * 1e-3) / 1e6


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self

        def run():
            for line in self.proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()
        return self

    def stop(self):
        if getattr(self, "proc", None):
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm = [float(s[1]) for s in self.samples if len(s) >= 9 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) >= 9 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            if len(s) >= 9:
                for k, nm in enumerate(names):
                    if s[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


def dram_traffic(kernel, n_cells):
    """DRAM bytes (read + write) per launch of `kernel`, from the committed ncu
    summary (profiles/dram_traffic_per_cell.txt: one 'kernel bytes_per_cell'
    line per kernel, dram__bytes_read.sum + dram__bytes_write.sum of one
    launch on this workload divided by its cells, scaled here by the cells one
    launch processes); None when absent."""
    path = os.path.join(ROOT, "profiles", "dram_traffic_per_cell.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) == 2 and parts[0] == kernel:
                return float(parts[1]) * n_cells
    except OSError:
        pass
    return None


def stage_bytes_per_cell(n_cells, n_faces, n_members):
    """The fixed two-kernel-minimum byte count per cell and RK stage of the
    whole stage (gradient + limiter kernel; flux + residual + update kernel),
    neighbour gathers counted once, boundary faces ignored, with the mesh's
    measured S (stencil members per cell) and Nf/Nc:
      FP64:  cv r/w 80 + rhsSum r/w 80 + gradients w/r 240 + vol 8 + cofg 24
             + R factor 48 + stencil ids 4 S + (fn 32 + fc 24 + f2c 8) Nf/Nc
      mixed: the same terms with FP32 gradients (120) and FP32 geometry
             (vol 4, cofg 12, R factor 24, face 16 + 12 + 8), the master cv
             and rhsSum counted in FP64 (80 + 80).
    At 128^3 hexes (S = 25.6, Nf/Nc = 2.98): 773 and 530 bytes."""
    s = n_members / n_cells
    r = n_faces / n_cells
    fp64 = 80 + 80 + 240 + 8 + 24 + 48 + 4 * s + 64 * r
    mixed = 80 + 80 + 120 + 4 + 12 + 24 + 4 * s + 36 * r
    return {"fp64": fp64, "mixed": mixed, "S": s, "nf_per_nc": r}


def algorithmic_bytes(region, precision):
    """Bytes per launch of the three stage kernels, counted from the data each
    kernel must move once (every cell or face record read once, neighbour
    re-reads and tile halos excluded).

    mixed (packed records, tiled gradient kernel):
      gradient+limiter  per cell: prim record 32, stencil offset 4, L matrix
                        24, face-entry offset 4, gradient record 64; per
                        stencil member: 2-byte local id; per cell-face entry
                        (2 nf + nb): 16-byte offset/neighbour entry
      face flux         per interior face: 48-byte record; per cell: prim 32 +
                        gradient 64; per face: 20 bytes of flux written; per
                        boundary face: 36 bytes of SoA geometry
      gather+update     per cell: cv read+write 80, p 8, prim record 32, 1/vol
                        4, centroid 12, CSR offset 4, rhsSum 80/3 (written in
                        stage 1, read+written in 2, read in 3); per face: flux
                        20; per cell-face entry: 4
    fp64 (structure of arrays, per-member LSQ weights)."""
    g = region.grid
    nc = region.n_cells
    nf = g.f2c.shape[0]
    nb = g.bf2c.shape[0]
    S = len(g.c2cs)
    ent = 2 * nf + nb
    if precision == "mixed":
        grad_limit = nc * (32 + 4 + 24 + 4 + 64) + S * 2 + ent * 16
        face_flux = nf * 48 + nc * 96 + (nf + nb) * 20 + nb * 36
        gather_update = nc * (80 + 8 + 32 + 4 + 12 + 4 + 80.0 / 3) + (nf + nb) * 20 + ent * 4
    else:
        r = 8
        grad_limit = nc * (5 * r + 15 * r + 4) + S * (4 + 3 * r) + nf * 2 * (8 + 3 * r)
        face_flux = nc * (5 * r + 15 * r) + (nf + nb) * (4 * r + 3 * r + 5 * r) + nf * 8
        gather_update = nc * (40 + 40 + 24 + 5 * 2 * r + 5 * r + 8 + 8) + 2 * nf * 5 * r + (2 * nf + nb) * 4
    return {"gradLimit": grad_limit, "faceFlux": face_flux, "gatherUpdate": gather_update}


def run_ours(args):
    import torch

    from rocflu_gb300 import cases, gpu

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    if args.only_adjoint:
        # the adjoint timing alone, on the single-VJP workload (profiling runs
        # of the adjoint kernels), for each precision in --precisions
        num = cases.Numerics(space_order=2, space_discr=cases.DISCR_ROE, reconst=args.adj_reconst)
        ac = cases.adjoint_tets(args.adj_n, num=num)
        out = {"reconst": args.adj_reconst}
        for prec in [x for x in args.precisions.split(",") if x]:
            areg = gpu.Region(ac, prec)
            at = areg.adjoint_times(3)
            out[prec] = {"primal_residual_ms": at[0], "vjp_ms": at[1], "vjp_over_primal": at[1] / at[0]}
            areg.close()
        if rank == 0:
            print(json.dumps({"partial": True, "adjoint": out}))
        return

    case = cases.shock_sphere(args.n)
    t0 = time.time()
    setup = gpu.Setup(case)
    setup_s = time.time() - t0
    # imposed first step = the CFL step of the initial state
    probe = gpu.Region(case, "fp64", grid=setup)
    case.num.dt_imposed = probe.timestep(1.0)
    probe.close()
    del probe

    results = {}
    regions = {}
    precs = [x for x in args.precisions.split(",") if x]
    clk = ClockSampler(local).start()
    for prec in precs:
        reg = gpu.Region(case, prec, grid=setup)
        regions[prec] = reg
        stream = torch.cuda.ExternalStream(reg.stream)
        t = 0.0
        n, t, rc = reg.step(args.warmup, t)
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        n, t, rc = reg.step(args.steps, t)
        e1.record(stream)
        e1.synchronize()
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1), dev)
        clocks = None
        units = region_units = reg.n_cells * reg.n_stages * args.steps
        results[prec] = {"ms": ms, "value": whole_job_value(units, ws, ms), "clocks": clocks, "rc": rc,
                         "time": t, "steps": n}
        ktimes = reg.kernel_times(5)
        results[prec]["kernel_ms"] = {"gradLimit": ktimes[0], "faceFlux": ktimes[1], "gatherUpdate": ktimes[2],
                                      "timestep": ktimes[3]}
        del region_units

    if set(precs) != {"mixed", "fp64"}:
        if rank == 0:
            print(json.dumps({"partial": True, "results": results}))
        return
    cv_m, _ = regions["mixed"].download(with_dv=False)

    # end-to-end through the C ABI with host buffers
    e2e = None
    if not args.skip_e2e:
        reg = regions["mixed"]
        host_cv = torch.empty((reg.n_cells, 5), dtype=torch.float64).pin_memory()
        cv_np = host_cv.numpy()
        cv_np[:] = cv_m
        t = 1.0
        # each step: cv host -> device (upload_state), one RungeKuttaMP step,
        # the new cv device -> host (download_state; dv is derived from cv)
        for _ in range(args.warmup):
            reg.upload(cv_np)
            _, t, _ = reg.step(1, t)
            reg.download(cv_np, with_dv=False)
        barrier()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            reg.upload(cv_np)
            _, t, _ = reg.step(1, t)
            reg.download(cv_np, with_dv=False)
        barrier()
        wall = max_over_ranks(time.perf_counter() - w0, dev)
        units = reg.n_cells * reg.n_stages * args.steps
        e2e = {"value": whole_job_value(units, ws, wall * 1e3), "unit": UNIT, "h2d_bytes_per_step": int(host_cv.numel() * 8),
               "d2h_bytes_per_step": int(host_cv.numel() * 8)}
    clocks = clk.stop()

    # mixed vs FP64 from the same initial state after the configured steps
    err = accuracy_run(regions, case, args.accuracy_steps)

    # roofline of the dominant kernel of the mixed path
    peaks, peak_kind = measured_peaks()
    ab = algorithmic_bytes(regions["mixed"], "mixed")
    km = results["mixed"]["kernel_ms"]
    dom = max(("gradLimit", "faceFlux", "gatherUpdate"), key=lambda k: km[k])
    achieved = ab[dom] / (km[dom] * 1e-3) / 1e9
    traffic = dram_traffic(dom, regions["mixed"].n_cells)
    roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": ab[dom], "launch_ms": km[dom]}

    # whole-stage roofline of both paths (fixed per-cell-stage formula)
    sb = stage_bytes_per_cell(regions["mixed"].n_cells, int(setup.f2c.shape[0]), int(setup.c2cs.shape[0]))
    stage_roof = {"formula": "stage_bytes_per_cell (bench.py)", "S": sb["S"], "nf_per_nc": sb["nf_per_nc"],
                  "peak_gbs": peaks["hbm_gbs"], "peak_source": peak_kind}
    for prec in ("mixed", "fp64"):
        stage_ms = results[prec]["ms"] / (args.steps * regions[prec].n_stages)
        ach = sb[prec] * regions[prec].n_cells / (stage_ms * 1e-3) / 1e9
        stage_roof[prec] = {"bytes_per_cell_stage": sb[prec], "stage_ms": stage_ms, "achieved_gbs": ach,
                            "frac": ach / peaks["hbm_gbs"]}

    fp64_tflops = gpu.fp64_rate()
    fp64 = {"value": results["fp64"]["value"], "ms_per_step": results["fp64"]["ms"] / args.steps,
            "kernel_ms": results["fp64"]["kernel_ms"], "mixed_over_fp64": results["mixed"]["value"] / results["fp64"]["value"],
            "mixed_vs_fp64_error": err,
            "roofline": {"bound": "fp64", "peak_fp64_tflops_measured": fp64_tflops,
                         "note": "FP64 kernels run the FP64 pipe at ~90% (ncu, profiles/); HBM is not their bound"}}

    # single-residual adjoint: 32^3 x 6 jittered tets, 2nd-order Roe,
    # componentwise Barth-Jespersen (crosses active limiter branches; the
    # reference's Venkatakrishnan factor jumps from 0 to 1 within
    # |d2| ~ 1e-9, far inside what an eps = 1e-6 difference resolves)
    adjoint = None
    if not args.skip_adjoint:
        adjoint = single_adjoint(args, cases, gpu)
        # the headline's limiter: Barth-Jespersen with the eigen-frame
        # velocity limiter (RECONST 10)
        adjoint["eigenframe"] = single_adjoint(args, cases, gpu, reconst=cases.RECONST_BJ, n_dirs=32)
        # the solver's default reconstruction: WENO-XYZ smoothing with the
        # simple limiter (RECONST 2)
        adjoint["weno_xyz"] = single_adjoint(args, cases, gpu, reconst=cases.RECONST_WENO_XYZ, n_dirs=32)
    unrolled = None if args.skip_unrolled else unrolled_adjoint(args, cases, gpu)
    weno = None if args.skip_weno else weno_variant(args, cases, gpu, setup, case.num.dt_imposed)
    tets = None if args.skip_tets else tet_block(args, cases, gpu)
    for reg in regions.values():
        reg.close()
    regions_cells = int(setup.n_cells)

    cpu = None
    if rank == 0 and not args.skip_cpu and ws == 1:
        cpu = cpu_sample(case, args.cpu_steps)
        cpu["gpu_over_cpu"] = {"mixed": results["mixed"]["value"] / cpu["value"],
                               "fp64": results["fp64"]["value"] / cpu["value"]}

    if rank == 0:
        ms = results["mixed"]["ms"]
        line = {
            "metric": METRIC, "value": results["mixed"]["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": workload_config(args.n, regions_cells, int(setup.f2c.shape[0]), ws),
            "setup_s": setup_s,
            # mixed step graph: step begin, gradient+dt, dt finalize, face flux and
            # gather-update of stage 1, three kernels per later stage, step end;
            # plus the one scalar-setting kernel of the step call
            "gpu_launches": 12 * args.steps + 1,
            "kernel_ms": results["mixed"]["kernel_ms"],
            "fp64": fp64,
            "adjoint": adjoint,
            "unrolled_adjoint": unrolled,
            "weno": weno,
            "tets": tets,
            "e2e": e2e,
            "roofline": roof,
            "stage_roofline": stage_roof,
            "cpu_baseline": cpu,
            "clocks": clocks,
        }
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def single_adjoint(args, cases, gpu, reconst=None, n_dirs=64):
    """One VJP of the residual and the gradient of J = sum_{x=1 patch} p_f |A_f|
    on the 32^3 x 6 jittered-tet case, FP64 and mixed: times, VJP/primal,
    and central differences (eps = 1e-6, FP64 residual) of J on seeded
    directions.  Each direction is classified by whether a cell of the
    functional's support (the cells owning the x=1 patch's faces, whose
    limited gradients alone enter the face pressures) changes its limiter's
    active branch (face or extreme neighbour) between U - eps v, U and
    U + eps v (rflu_gpu_limiter_branches): the functional is smooth along
    the others, which the adjoint must match to 1e-6.  Switches anywhere in
    the mesh are counted too.  A second pass at eps = 1e-8 repeats the
    classification with fewer kinks crossed."""
    if reconst is None:
        reconst = cases.RECONST_BJ_COMP
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_ROE, reconst=reconst)
    ac = cases.adjoint_tets(args.adj_n, num=num)
    areg, mreg = gpu.Region(ac, "fp64"), gpu.Region(ac, "mixed")
    tag = {cases.RECONST_BJ_COMP: "bjcomp", cases.RECONST_BJ: "bj_eigenframe", cases.RECONST_VENKAT: "venkat",
           cases.RECONST_WENO_XYZ: "wenoxyz"}[reconst]
    out = {"workload": "adjoint_tets%d_roe_%s" % (args.adj_n, tag), "cells": areg.n_cells,
           "functional": "sum_{x=1 patch} p_f |A_f|"}
    rng = np.random.default_rng(2)
    scale = np.abs(ac.cv0).mean(axis=0)
    dirs = [rng.standard_normal(ac.cv0.shape) * scale for _ in range(n_dirs)]
    g = areg.grid
    support = np.unique(g.bf2c[g.patch_off[1]:g.patch_off[2]] - 1)
    b0 = areg.limiter_branches(ac.cv0)

    def differences(eps):
        fd, switch, switch_all = [], [], []
        for v in dirs:
            jp, _ = areg.patch_pressure(ac.cv0 + eps * v, 1, with_grad=False)
            jm, _ = areg.patch_pressure(ac.cv0 - eps * v, 1, with_grad=False)
            fd.append((jp - jm) / (2 * eps))
            bp, bm = areg.limiter_branches(ac.cv0 + eps * v), areg.limiter_branches(ac.cv0 - eps * v)
            changed = (bp != b0).any(axis=2) | (bm != b0).any(axis=2)
            switch.append(int(changed[support].sum()))
            switch_all.append(int(changed.sum()))
        return np.array(fd), np.array(switch), np.array(switch_all)

    eps = 1e-6
    fd, switch, switch_all = differences(eps)
    smooth = switch == 0
    # the same at eps = 1e-8: fewer directions cross a kink, at the price of
    # the difference's rounding (about 1e-16 |J| / eps)
    eps_s = 1e-8
    fd_s, switch_s, _ = differences(eps_s)
    smooth_s = switch_s == 0
    lam = np.random.default_rng(5).standard_normal(ac.cv0.shape)
    g_ref = None
    for name, reg in (("fp64", areg), ("mixed", mreg)):
        at = reg.adjoint_times(5)
        J, gJ = reg.patch_pressure(ac.cv0, 1)
        err = np.abs(fd - np.array([(gJ * v).sum() for v in dirs])) / np.abs(fd)
        g = reg.vjp(ac.cv0, lam)
        res = {"primal_residual_ms": at[0], "vjp_ms": at[1], "vjp_over_primal": at[1] / at[0], "J": J,
               "fd_eps": eps, "fd_dirs": len(err), "fd_rel_err_median": float(np.median(err)),
               "fd_rel_err_max": float(err.max()), "fd_dirs_below_1e-6": int((err < 1e-6).sum()),
               "fd_dirs_below_1e-5": int((err < 1e-5).sum()),
               "branch_switch": {"dirs_without_switch": int(smooth.sum()),
                                 "without_switch_below_1e-6": int((err[smooth] < 1e-6).sum()),
                                 "without_switch_err_max": float(err[smooth].max()) if smooth.any() else None,
                                 "with_switch": int((~smooth).sum()),
                                 "with_switch_below_1e-6": int((err[~smooth] < 1e-6).sum()),
                                 "switching_support_cell_variables_median": float(np.median(switch[~smooth]))
                                 if (~smooth).any() else None,
                                 "support_cells": int(len(support)),
                                 "switching_cell_variables_anywhere_median": float(np.median(switch_all))}}
        err_s = np.abs(fd_s - np.array([(gJ * v).sum() for v in dirs])) / np.abs(fd_s)
        res["fd_small_eps"] = {"fd_eps": eps_s, "fd_rel_err_median": float(np.median(err_s)),
                               "dirs_without_switch": int(smooth_s.sum()),
                               "without_switch_below_1e-6": int((err_s[smooth_s] < 1e-6).sum()),
                               "without_switch_err_max": float(err_s[smooth_s].max()) if smooth_s.any() else None,
                               "with_switch_below_1e-6": int((err_s[~smooth_s] < 1e-6).sum())}
        if g_ref is None:
            g_ref = g
            out.update(res)
        else:
            res["vjp_rel_l2_diff_vs_fp64"] = float(np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref))
            res["vjp_over_fp64_primal"] = at[1] / out["primal_residual_ms"]
            out["mixed"] = res
    areg.close()
    mreg.close()
    return out


def weno_variant(args, cases, gpu, setup, dt_imposed):
    """The headline workload with the solver's default reconstruction instead
    of the BJ limiter: WENO-XYZ gradient smoothing + the simple positivity
    limiter (RECONST 2), HLLC, Wray RK3, mixed and FP64: step rate, the
    gradient phase (raw gradients + smoothing) per stage, and the mixed
    path's density error against the FP64 one after the same steps."""
    import torch

    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_WENO_XYZ, cfl=0.4)
    c = cases.shock_sphere(args.n, num=num)
    c.num.dt_imposed = dt_imposed
    steps, warm = 10, 3
    out = {"workload": "shock_sphere_hex%d_hllc_wenoxyz_wray3" % args.n, "steps": steps, "warmup": warm}
    cvs = {}
    for prec in ("mixed", "fp64"):
        reg = gpu.Region(c, prec, grid=setup)
        stream = torch.cuda.ExternalStream(reg.stream)
        _, t, _ = reg.step(warm, 0.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, t, rc = reg.step(steps, t)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        kt = reg.kernel_times(5)
        out[prec] = {"value": reg.n_cells * reg.n_stages * steps / (ms * 1e-3) / 1e6, "unit": UNIT,
                     "ms_per_step": ms / steps, "gradient_ms": kt[0], "face_flux_ms": kt[1], "update_ms": kt[2],
                     "rc": rc}
        cvs[prec] = reg.download()[0]
        reg.close()
    out["mixed_vs_fp64_L1_rho"] = float(np.abs(cvs["mixed"][:, 0] - cvs["fp64"][:, 0]).mean())
    return out


def unrolled_adjoint(args, cases, gpu):
    """Time-unrolled adjoint: spherical blast on n^3 hexes (p=10 inside
    r=0.15, p=1 outside, rho=1), HLLC, second order with the Barth-Jespersen
    limiter and its eigen-frame velocity limiting (RECONST 10; the
    reference's Venkatakrishnan limiter, whose face offsets are taken as
    cofg - fc, lets face pressures of this blast go negative within the
    first step), Wray RK3, dt fixed from the initial
    CFL 0.4, the functional the time-integrated pressure on the x=1 patch.  Gradient w.r.t. the initial
    density by the checkpointed reverse sweep; central differences on seeded
    density blobs, on the case as stated and on the same case with a smooth
    2% background variation.  As stated, the blast front does not reach the
    x=1 patch in 200 steps and a density change at rest under uniform
    pressure is a stationary contact, so J = steps * dt * p_ambient * area
    exactly and its gradient is ~0, checked in absolute terms; the smooth
    variant is the one whose differences test the adjoint."""
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ, cfl=0.4)
    c = cases.blast_hex(args.unrolled_n, num=num, p_in=10.0, radius=0.15)
    x = gpu.Setup(c).cofg
    reg = gpu.Region(c, "fp64")
    dt = reg.timestep(1.0)
    n, every = args.unrolled_steps, args.unrolled_every
    out = {"workload": "blast_hex%d_hllc_bj_wray3" % args.unrolled_n, "cells": reg.n_cells, "steps": n,
           "checkpoint_every": every, "dt": dt, "functional": "sum_n dt * sum_{x=1 patch} p_f |A_f|"}
    bg = np.sin(2 * np.pi * x[:, 0] + 0.3) * np.sin(2 * np.pi * x[:, 1] + 0.7) * np.sin(2 * np.pi * x[:, 2] + 1.1)
    smooth = c.cv0.copy()
    smooth[:, 0] *= 1 + 0.02 * bg
    smooth[:, 4] *= 1 + 0.02 * np.roll(bg, 7)
    smooth[:, 1] += 0.01 * bg
    # density blobs (sigma 0.1) between the blast and the x=1 wall, where the
    # functional has a sensitivity well above the differences' round-off
    rng = np.random.default_rng(2024)
    dirs = []
    for _ in range(args.unrolled_fd):
        c0 = np.array([rng.uniform(0.55, 0.85), rng.uniform(0.3, 0.7), rng.uniform(0.3, 0.7)])
        d = np.zeros_like(c.cv0)
        d[:, 0] = np.exp(-((x - c0) ** 2).sum(axis=1) / (2 * 0.1 ** 2)) * rng.choice([-1.0, 1.0])
        dirs.append(d)
    for name, cv0, epss, ndir in (("as_stated", c.cv0, (1e-4,), 4),
                                  ("smooth_background", smooth, (1e-4, 1e-5), len(dirs))):
        reg.upload(cv0)
        J, g, st = reg.unrolled_adjoint(cv0, n, dt, every, 1)
        res = {"J": J, "grad_abs_max": float(np.abs(g).max()), "grad_finite": bool(np.isfinite(g).all()),
               "forward_ms": st["forward_ms"], "reverse_ms": st["reverse_ms"],
               "adjoint_over_primal": st["reverse_ms"] / st["forward_ms"],
               "device_bytes": st["device_bytes"], "checkpoints": st["checkpoints"], "fd": []}
        if name == "as_stated":
            # a stationary contact: J is steps * dt * p_ambient * (patch area)
            # and its gradient vanishes, so the check is absolute: J against
            # that closed form, and both the differences and the adjoint's
            # directional derivatives against J's rounding
            area = 1.0
            p_amb = 1.0
            fds, ads = [], []
            for d in dirs[:ndir]:
                jp, _, _ = reg.unrolled_adjoint(cv0 + 1e-4 * d, n, dt, every, 1, with_grad=False)
                jm, _, _ = reg.unrolled_adjoint(cv0 - 1e-4 * d, n, dt, every, 1, with_grad=False)
                fds.append(abs((jp - jm) / 2e-4))
                ads.append(abs(float((g * d).sum())))
            res["closed_form"] = {"J_expected": n * dt * p_amb * area, "J_rel_diff": abs(J - n * dt * p_amb * area) / J,
                                  "fd_eps": 1e-4, "dirs": ndir, "fd_abs_max": float(max(fds)),
                                  "ad_abs_max": float(max(ads)), "J_rounding_over_eps": float(J * 1e-16 / 1e-4)}
            out[name] = res
            continue
        for eps in epss:  # relative density change at a blob's centre
            errs, absd = [], []
            for d in dirs[:ndir]:
                jp, _, _ = reg.unrolled_adjoint(cv0 + eps * d, n, dt, every, 1, with_grad=False)
                jm, _, _ = reg.unrolled_adjoint(cv0 - eps * d, n, dt, every, 1, with_grad=False)
                ad = float((g * d).sum())
                fd = (jp - jm) / (2 * eps)
                absd.append(abs(ad))
                errs.append(abs(fd - ad) / max(abs(ad), 1e-300))
            errs = np.array(errs)
            ok = np.isfinite(errs)
            res["fd"].append({"eps": eps, "dirs": len(errs), "rel_err_median": float(np.median(errs[ok])) if ok.any() else None,
                              "rel_err_max": float(errs[ok].max()) if ok.any() else None,
                              "below_1e-6": int((errs < 1e-6).sum()), "below_1e-5": int((errs < 1e-5).sum()),
                              "below_1e-4": int((errs < 1e-4).sum()), "not_finite": int((~ok).sum()),
                              "ad_abs_median": float(np.median(absd))})
        if name == "smooth_background":
            # the same gradient with the mixed primal and mixed stage VJPs
            mreg = gpu.Region(c, "mixed")
            Jm, gm, stm = mreg.unrolled_adjoint(cv0, n, dt, every, 1)
            res["mixed"] = {"J": Jm, "forward_ms": stm["forward_ms"], "reverse_ms": stm["reverse_ms"],
                            "adjoint_over_primal": stm["reverse_ms"] / stm["forward_ms"],
                            "reverse_speedup_vs_fp64": st["reverse_ms"] / stm["reverse_ms"],
                            "device_bytes": stm["device_bytes"],
                            "grad_rel_l2_diff_vs_fp64": float(np.linalg.norm(gm - g) / np.linalg.norm(g)),
                            "grad_rel_max_diff_vs_fp64": float(np.abs(gm - g).max() / np.abs(g).max())}
            mreg.close()
        out[name] = res
    reg.close()
    return out


def workload_config(n, cells, faces, ws):
    """The config block both arms print for the headline workload."""
    return {"workload": "shock_sphere_hex%d_hllc_bj_wray3" % n, "cells": int(cells), "faces": int(faces),
            "stages_per_step": 3, "flux": "HLLC", "limiter": "BJ (RECONST 10)",
            "parallelism": "replicas" if ws > 1 else "single", "l2": "working set > L2 (no flush)"}


def accuracy_run(regions, case, n_steps, marks=(100, 250)):
    """The mixed path against the FP64 path from the same initial state:
    L1/Linf of density and pressure after each mark and after n_steps whole
    steps (CFL time step each step; the imposed first step is the CFL step
    of the initial state)."""
    for r in regions.values():
        r.upload(case.cv0)
    t = {k: 0.0 for k in regions}
    rcs = {k: 0 for k in regions}
    done = 0
    hist = []
    for m in sorted({x for x in marks if x < n_steps} | {n_steps}):
        for k, r in regions.items():
            n, t[k], rc = r.step(m - done, t[k])
            rcs[k] |= rc
        cvm, dvm = regions["mixed"].download()
        cvd, dvd = regions["fp64"].download()
        hist.append({"steps": m, "L1_rho": float(np.abs(cvm[:, 0] - cvd[:, 0]).mean()),
                     "Linf_rho": float(np.abs(cvm[:, 0] - cvd[:, 0]).max()),
                     "L1_p": float(np.abs(dvm[:, 0] - dvd[:, 0]).mean()),
                     "Linf_p": float(np.abs(dvm[:, 0] - dvd[:, 0]).max()),
                     "time_mixed": t["mixed"], "time_fp64": t["fp64"]})
        done = m
    out = dict(hist[-1])
    out["history"] = hist
    out["event_codes"] = rcs
    out["status"] = {k: r.status() for k, r in regions.items()}
    return out


def tet_block(args, cases, gpu):
    """Throughput on the tetrahedral blast mesh of the 3-D blast
    configuration: 64^3 hexes split into 6 jittered tetrahedra (1,572,864
    cells, seed 0), HLLC, second order, Wray RK3, CFL 0.4, slip walls, at
    p = 4 inside r < 0.1, with the Barth-Jespersen limiter (RECONST 10).  In
    the reference scheme the configuration's p = 100 drives face pressures
    negative within a few steps with every limiter, and at p = 4 the
    Venkatakrishnan limiter gives non-finite cells from step 5 on (the CPU
    oracle and the FP64 device path alike); Barth-Jespersen carries p = 4
    cleanly.  Mixed and FP64 step rates and each one's whole-stage roofline
    with this mesh's measured S (stencil members per cell) and Nf/Nc."""
    import torch

    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ, cfl=0.4)
    c = cases.blast_tets(args.tet_n, num=num, p_in=4.0)
    t0 = time.time()
    setup = gpu.Setup(c)
    setup_s = time.time() - t0
    probe = gpu.Region(c, "fp64", grid=setup)
    c.num.dt_imposed = probe.timestep(1.0)
    probe.close()
    nc, nf, nnz = int(setup.n_cells), int(setup.f2c.shape[0]), int(setup.c2cs.shape[0])
    sb = stage_bytes_per_cell(nc, nf, nnz)
    peaks, peak_kind = measured_peaks()
    steps, warm = 10, 3
    out = {"workload": "blast_tets%dx6_hllc_bj_wray3_p4" % args.tet_n, "cells": nc, "faces": nf,
           "boundary_faces": int(setup.bf2c.shape[0]), "S": sb["S"], "nf_per_nc": sb["nf_per_nc"],
           "steps": steps, "warmup": warm, "setup_s": setup_s, "peak_gbs": peaks["hbm_gbs"], "peak_source": peak_kind}
    for prec in ("mixed", "fp64"):
        reg = gpu.Region(c, prec, grid=setup)
        stream = torch.cuda.ExternalStream(reg.stream)
        _, t, _ = reg.step(warm, 0.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, t, rc = reg.step(steps, t)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        kt = reg.kernel_times(5)
        stage_ms = ms / (steps * reg.n_stages)
        ach = sb[prec] * nc / (stage_ms * 1e-3) / 1e9
        st = reg.status()
        out[prec] = {"value": nc * reg.n_stages * steps / (ms * 1e-3) / 1e6, "unit": UNIT, "ms_per_step": ms / steps,
                     "kernel_ms": {"gradLimit": kt[0], "faceFlux": kt[1], "gatherUpdate": kt[2], "timestep": kt[3]},
                     "stage_roofline": {"bytes_per_cell_stage": sb[prec], "stage_ms": stage_ms, "achieved_gbs": ach,
                                        "frac": ach / peaks["hbm_gbs"]},
                     "rc": rc, "nanCells": st["nanCells"], "posFixCells": st["posFixCells"], "time": t}
        reg.close()
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def _oracle_case(n):
    """The headline workload for the CPU oracle, with the imposed first step
    set, as on the device, to the CFL step of the initial state."""
    from oracle import oracle as orc
    from rocflu_gb300 import cases

    case = cases.shock_sphere(n)
    o = orc.Oracle(case)
    o.set_dt_imposed(o.timestep(1.0))
    return case, o


def cpu_sample(case, n_steps):
    """The CPU oracle (FP64 restatement of the reference path, OpenMP over
    every host core) on the same 128^3 workload: one untimed step (the
    imposed first step), n_steps timed whole steps on all cores, then one
    step on one thread."""
    from oracle import oracle as orc

    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    t0 = time.perf_counter()
    o = orc.Oracle(case)
    o.set_dt_imposed(case.num.dt_imposed)
    setup_s = time.perf_counter() - t0
    _, t = o.run(1, 0.0)
    t0 = time.perf_counter()
    _, t = o.run(n_steps, t)
    el = time.perf_counter() - t0
    units = o.n_cells * o.n_stages() * n_steps
    orc.set_threads(1)
    t0 = time.perf_counter()
    _, t = o.run(1, t)
    el1 = time.perf_counter() - t0
    orc.set_threads(cores)
    return {"value": units / el / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "the same %d-cell mesh and set-up, %d whole Wray steps after one untimed step, %d threads, "
                      "%.1f s (oracle set-up %.1f s untimed)" % (o.n_cells, n_steps, cores, el, setup_s),
            "single_thread": {"value": o.n_cells * o.n_stages() / el1 / 1e6, "unit": UNIT, "cores": 1,
                              "sample": "one whole step of the same workload, %.1f s" % el1}}


def run_reference(args):
    """The reference arm: the CPU restatement of the reference path (the
    Fortran reference cannot be built here or on the GPU machine) on the same
    128^3 workload with every host core; each bench step is one whole time
    step (CFL time step + three Wray stages), W untimed, K timed."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from oracle import oracle as orc

    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    t0 = time.perf_counter()
    case, o = _oracle_case(args.n)
    setup_s = time.perf_counter() - t0
    t = 0.0
    for _ in range(args.warmup):
        _, t = o.run(1, t)
    els = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, t = o.run(1, t)
        els.append(time.perf_counter() - t0)
    total = sum(els)
    value = o.n_cells * o.n_stages() * args.steps / total / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.n, o.n_cells, o.n_faces, ws),
            "setup_s": setup_s,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "the FP64 CPU restatement of the reference path (OpenMP, %d threads) on the "
                                       "same %d-cell mesh: %d whole Wray steps after %d untimed"
                                       % (cores, o.n_cells, args.steps, args.warmup)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
