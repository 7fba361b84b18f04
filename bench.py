#!/usr/bin/env python3
"""Benchmark of the stair-step weighted-Jacobi solve (the reference's
bandwidth benchmark) on a GB300.

Workload (default, 'jacobi256'): 256^3 stretched grid (geometric ratio 1.01),
four seeded blocked boxes of 8-40 cells per side (one touching the outer
boundary), the phi_x influence problem (body_grad = e_x, zero outer data,
compatibility applied), exactly 2000 weighted-Jacobi sweeps (tolerance < 0,
one residual check at the end), gauge and final residual.  A step is one full
solve_stairstep_poisson_3d call.

  value  whole-job algorithmic HBM throughput, 32 B/cell/sweep (read phi, src,
         rdiag; write phi'), device-resident inputs, CUDA events on the
         solver's stream
  e2e    the same metric through the host-array C ABI call (pinned host
         buffers; host->device upload of every input and device->host copy of
         phi inside the timed region)

--impl reference times the CPU oracle (the reference's algorithm restated in
C, OpenMP over z-planes, every host core) on a bounded sample of the same
workload: the oracle is the reference arm because the reference itself is
Fortran/OpenACC and no Fortran compiler is available.

Other workloads (one GPU, a JSON line each):
  pcg_sphere      sphere on 64x64x32 and
  pcg_ellipsoids  3 ellipsoids on 384x384x192: phi_x, phi_y, phi_z to a 1e-10
                  max-norm residual with plain FP64 PCG, FP32 PCG in FP64
                  refinement (diagonal and multigrid preconditioners) and the
                  learned initial guess; value is the multigrid arm's solve time
  foil_frames     256 uneven 2-D foil frames, two potentials and the four
                  partition terms each
  learned_guess   the trained network as initial guess on unseen bodies

Multi-GPU: replicas only (each rank solves its own copy; no collective on the
data path); value is the sum over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_CELL_SWEEP = 32
SWEEPS = 2000
METRIC = "Jacobi HBM GB/s (weighted-Jacobi stair-step solve, 32 B/cell/sweep)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=256, help="grid size per axis (default 256)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--method", choices=["jacobi_fma", "jacobi_tf", "jacobi", "jacobi_df"], default="jacobi_fma",
                    help="jacobi256: the sweep timed as the headline (the others are timed as secondary keys)")
    ap.add_argument("--head-only", action="store_true", help="jacobi256: time only the headline method")
    ap.add_argument("--no-pcg", action="store_true",
                    help="jacobi256: skip the three-potential PCG measurement on the 384x384x192 grid")
    ap.add_argument("--no-densities", action="store_true",
                    help="pcg_sphere / pcg_ellipsoids: skip the force densities on the solved potentials")
    ap.add_argument("--grid", type=int, nargs=3, default=None,
                    help="pcg_ellipsoids / densities: a smaller grid of the same generator (profiling runs)")
    ap.add_argument("--frames", type=int, default=256,
                    help="foil_frames: the first N frames of the 256-frame generator (profiling runs)")
    ap.add_argument("--arms", default="fp64,mixed,mg,learned_mixed,learned_mg",
                    help="pcg_sphere / pcg_ellipsoids: comma-separated solver arms to time (profiling runs take "
                         "one); learned_guess: add fcg_learned for the flexible CG with the network")
    ap.add_argument("--workload", choices=["jacobi256", "pcg_sphere", "pcg_ellipsoids", "foil_frames", "learned_guess",
                                           "densities"],
                    default="jacobi256",
                    help="jacobi256: the headline bandwidth benchmark; pcg_sphere / pcg_ellipsoids: three-potential PCG "
                         "time to 1e-10 (plain FP64 vs mixed precision)")
    return ap.parse_args()


def workload(n):
    from flowfpmpp_gb300 import workloads
    return workloads.boxes_grid(n=n)


def config(n, method="jacobi_fma"):
    return {"workload": f"stair-step weighted Jacobi {n}^3, 4 boxes, phi_x, {SWEEPS} sweeps",
            "grid": [n, n, n], "sweeps": SWEEPS, "method": method, "stretch_ratio": 1.01,
            "l2_policy": "inputs larger than L2 (phi, src, rdiag, phi' = 4 x 134 MB per sweep)"}


def algorithmic_gb(n, sweeps=SWEEPS):
    return BYTES_PER_CELL_SWEEP * float(n) ** 3 * sweeps / 1e9


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""
        return False

    def summary(self):
        if self.proc is None:
            return None
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm, smax = float(parts[1]), float(parts[2])
            except ValueError:
                continue
            sms.append(sm)
            mx = smax
            for nm, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sms)}


# ---------------------------------------------------------------- CPU side
def cpu_sample(n, budget_s=12.0, threads=None):
    """Oracle sweeps on the host cores: returns (GB/s, cores, sweeps, seconds)."""
    import oracle as orc
    f = workload(n)
    faces = [a.copy(order="F") for a in f["faces"]]
    orc.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], f["body"], *faces, f["dx"], f["dy"], f["dz"])
    coefs = orc.stairstep_coefficients(f["xc"], f["yc"], f["zc"], f["dx"], f["dy"], f["dz"])
    src, diag, rdiag, iso = orc.build_operator(f["rhs"], f["solid"], f["body"], *faces, coefs, f["dx"], f["dy"],
                                               f["dz"], False)
    a = f["phi"].copy(order="F")
    b = a.copy(order="F")
    cores = threads or orc.max_threads()
    orc.set_threads(cores)
    orc.jacobi_sweep(a, b, src, rdiag, coefs)  # warm
    t0 = time.perf_counter()
    sweeps = 0
    while True:
        for _ in range(5):
            orc.jacobi_sweep(a, b, src, rdiag, coefs)
            a, b = b, a
        sweeps += 5
        el = time.perf_counter() - t0
        if el >= budget_s or sweeps >= SWEEPS:
            break
    orc.set_threads(1)
    return BYTES_PER_CELL_SWEEP * float(n) ** 3 * sweeps / el / 1e9, cores, sweeps, el


def run_reference(args):
    """The reference arm: the CPU oracle on every host core, each step a
    bounded sample (sweeps) of the same 2000-sweep workload."""
    n = args.n
    import oracle as orc
    orc.build()
    f = workload(n)
    faces = [a.copy(order="F") for a in f["faces"]]
    orc.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], f["body"], *faces, f["dx"], f["dy"], f["dz"])
    coefs = orc.stairstep_coefficients(f["xc"], f["yc"], f["zc"], f["dx"], f["dy"], f["dz"])
    src, diag, rdiag, iso = orc.build_operator(f["rhs"], f["solid"], f["body"], *faces, coefs, f["dx"], f["dy"],
                                               f["dz"], False)
    cores = orc.max_threads()
    orc.set_threads(cores)
    a = f["phi"].copy(order="F")
    b = a.copy(order="F")
    per_step = 20  # sweeps per step: a bounded sample of the 2000-sweep solve
    for _ in range(args.warmup):
        for _ in range(per_step):
            orc.jacobi_sweep(a, b, src, rdiag, coefs)
            a, b = b, a
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for _ in range(per_step):
            orc.jacobi_sweep(a, b, src, rdiag, coefs)
            a, b = b, a
    el = time.perf_counter() - t0
    gbs = BYTES_PER_CELL_SWEEP * float(n) ** 3 * per_step * args.steps / el / 1e9
    sample = f"{per_step} weighted-Jacobi sweeps of the {n}^3 operator per step (oracle, OpenMP over z-planes)"
    line = {"metric": METRIC, "value": gbs, "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded boxes)",
            "config": config(n), "impl": "reference",
            "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- PCG time to solution
def run_pcg(args):
    """Three influence potentials (phi_x, phi_y, phi_z) to a 1e-10 max-norm
    residual: plain FP64 PCG (one after the other, the reference's method),
    FP32 PCG in FP64 refinement batched over the three right-hand sides
    (diagonal preconditioner), the same refinement with the multigrid
    preconditioner, and both with the learned initial guess."""
    import torch
    from flowfpmpp_gb300 import build as fbuild
    fbuild.build()
    import flowfpmpp_gb300
    from flowfpmpp_gb300 import stairstep as ss
    from flowfpmpp_gb300 import workloads
    lib = flowfpmpp_gb300.lib()
    if args.workload == "pcg_sphere":
        f = workloads.sphere_grid()
        name = "sphere 64x64x32, ratio 1.03"
    elif args.grid:
        f = workloads.ellipsoids_grid(*args.grid)
        name = "3 ellipsoids %dx%dx%d, ratio 1.02" % tuple(args.grid)
    else:
        f = workloads.ellipsoids_grid()
        name = "3 ellipsoids 384x384x192, ratio 1.02"
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
    faces_dev, bgs, rhss = [], [], []
    for axis in range(3):
        body = np.zeros(3)
        body[axis] = 1.0
        faces = [x.copy(order="F") for x in f["faces"]]
        ss.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], body, *faces, f["dx"], f["dy"], f["dz"])
        faces_dev += [dev(x) for x in faces]
        bgs.append(body)
        rhss.append(dev(f["rhs"]))
    phis = [dev(f["phi"]) for _ in range(3)]
    dsolid = dev(f["solid"])
    dax = [dev(f[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    VP = ctypes.c_void_p
    bg = np.ascontiguousarray(np.concatenate(bgs))
    stream = torch.cuda.current_stream()

    from flowfpmpp_gb300 import learned as lg
    net = lg.LearnedGuess.load() if os.path.exists(lg.WEIGHTS) and nx % 8 == 0 and ny % 8 == 0 and nz % 8 == 0 \
        else None
    fallbacks = (ctypes.c_int * 3)()

    def solve(method, use_net=False):
        for t in phis:
            t.zero_()
        sweeps = (ctypes.c_int * 3)()
        res = (ctypes.c_double * 3)()
        args_ = (3, (VP * 3)(*[t.data_ptr() for t in phis]), (VP * 3)(*[t.data_ptr() for t in rhss]),
                 VP(dsolid.data_ptr()), bg.ctypes.data_as(VP), (VP * 18)(*[t.data_ptr() for t in faces_dev]),
                 *[VP(t.data_ptr()) for t in dax], nx, ny, nz, ctypes.c_double(1e-10), 2000000, 50, method, sweeps,
                 res)
        if use_net:
            rc = lib.fpm_solve_stairstep_learned_dev(net.h, *args_, fallbacks, VP(stream.cuda_stream))
        else:
            rc = lib.fpm_solve_stairstep_multi_dev(*args_, VP(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fpm_last_error().decode())
        return list(sweeps), list(res)

    out = {}
    arms = [(0, "fp64", False), (3, "mixed", False), (4, "mg", False)]
    if net is not None:
        arms += [(3, "learned_mixed", True), (4, "learned_mg", True)]
    wanted = set(args.arms.split(","))
    arms = [a for a in arms if a[1] in wanted]
    for method, label, use_net in arms:
        for _ in range(args.warmup):
            solve(method, use_net)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            sw, res = solve(method, use_net)
        e1.record(stream)
        torch.cuda.synchronize()
        out[label] = {"seconds": e0.elapsed_time(e1) / args.steps / 1e3, "iterations": sw, "residual": res,
                      "phi": [t.cpu().numpy().copy() for t in phis]}
        if use_net:
            out[label]["fallbacks"] = list(fallbacks)
    head = "mg" if "mg" in out else next(iter(out))
    line = {"metric": "PCG solve time to 1e-10 max-norm residual, three potentials (FP32 PCG in FP64 refinement "
                      "with a multigrid preconditioner vs plain FP64 PCG)",
            "value": out[head]["seconds"], "unit": "s", "higher_is_better": False, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "data": "synthetic (seeded)",
            "config": {"workload": name, "grid": [nx, ny, nz], "rhs": 3, "tolerance": 1e-10, "check_interval": 50,
                       "arm": head}}
    for label in ("fp64", "mixed", "mg", "learned_mixed", "learned_mg"):
        if label not in out:
            continue
        lm = out[label]
        line[label] = {k: v for k, v in lm.items() if k != "phi"}
        if label != "fp64" and "fp64" in out:
            line[label]["speedup_vs_fp64"] = out["fp64"]["seconds"] / lm["seconds"]
            line[label]["vs_fp64_rel_linf"] = max(
                float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
                for a, b in zip(lm["phi"], out["fp64"]["phi"]))
    if not args.no_densities:
        line["densities"] = densities(args, lib, f, out, head, dsolid, dax, faces_dev, bgs, stream)
        for label, errs in line["densities"].pop("terms_vs_fp64").items():
            line[label]["terms_vs_fp64"] = errs
    print(json.dumps(line), flush=True)


def densities(args, lib, f, out, head, dsolid, dax, faces_dev, bgs, stream):
    """The force densities of every arm's three potentials in the C1 flow
    (U = 1 plus 8 Gaussian z-tubes, acceleration of 6 Fourier modes):
    -(omega x u).grad(phi_i), -a.grad(phi_i) and their integrals through
    fpm_compute_stairstep_fpm_terms_3d_dev, the call timed on the head arm's
    potentials (124 bytes per cell and potential: phi, nine flow fields and
    the solid flag read, five fields written), and each arm's integrals and
    density fields against the FP64 arm's."""
    import torch
    from flowfpmpp_gb300 import workloads
    VP = ctypes.c_void_p
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    fl = workloads.flow_c1(f)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
    dflow = [dev(fl[k]) for k in ("u", "v", "w", "ox", "oy", "oz", "ax", "ay", "az")]
    n3 = nx * ny * nz
    outs = [torch.empty(n3, dtype=torch.float64, device="cuda") for _ in range(5)]
    bounds = np.array([-1e300, 1e300] * 3)

    def terms(phi_t, axis):
        tot = (ctypes.c_double * 2)()
        bg = np.ascontiguousarray(bgs[axis], dtype=np.float64)
        rc = lib.fpm_compute_stairstep_fpm_terms_3d_dev(
            VP(phi_t.data_ptr()), *[VP(t.data_ptr()) for t in dflow], VP(dsolid.data_ptr()), bg.ctypes.data_as(VP),
            *[VP(t.data_ptr()) for t in dax], *[VP(t.data_ptr()) for t in faces_dev[6 * axis:6 * axis + 6]],
            bounds.ctypes.data_as(VP), *[VP(o.data_ptr()) for o in outs], tot, nx, ny, nz, VP(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fpm_last_error().decode())
        return [tot[0], tot[1]]

    ref, errs, head_totals, seconds = None, {}, None, None
    order = sorted(out, key=lambda lb: lb != "fp64")  # the FP64 arm first: the others are compared with it
    for label in order:
        phis = [torch.from_numpy(p).cuda() for p in out[label]["phi"]]
        r = []
        for axis in range(3):
            tot = terms(phis[axis], axis)
            r.append((tot, outs[3].cpu().numpy(), outs[4].cpu().numpy()))
        if label == "fp64":
            ref = r
        elif ref is not None:
            # integrals relative to the largest FP64 integral (some are zero by symmetry)
            scale = max(max(abs(x) for x in t0) for t0, _, _ in ref) or 1e-300
            tot_rel, field_rel = 0.0, 0.0
            for (t, vo, ad), (t0, vo0, ad0) in zip(r, ref):
                for a, b in zip(t, t0):
                    tot_rel = max(tot_rel, abs(a - b) / scale)
                for a, b in ((vo, vo0), (ad, ad0)):
                    field_rel = max(field_rel, float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)))
            errs[label] = {"integrals_rel": tot_rel, "densities_rel_linf": field_rel}
        if label == head:
            head_totals = [x[0] for x in r]
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = 5
            e0.record(stream)
            for _ in range(reps):
                for axis in range(3):
                    terms(phis[axis], axis)
            e1.record(stream)
            torch.cuda.synchronize()
            seconds = e0.elapsed_time(e1) / reps / 1e3
    gbs = 124.0 * n3 * 3 / seconds / 1e9
    return {"kernel": "k_terms", "seconds_three_potentials": seconds, "gbs": gbs, "bytes_per_cell_potential": 124,
            "integrals_head": head_totals, "terms_vs_fp64": errs}


def run_learned(args):
    """The committed trained network on unseen random bodies at 256x256x128
    (the training set was 128x128x64): FP64 PCG to 1e-10 from phi = 0 and from
    the learned initial guess, the multigrid-preconditioned refinement from
    phi = 0 and from the guess, and (with --arms naming fcg_learned) the
    flexible CG with the network as preconditioner; iterations, time and
    fallbacks over `steps` bodies (after `warmup` bodies)."""
    import torch
    from flowfpmpp_gb300 import build as fbuild
    fbuild.build()
    from flowfpmpp_gb300 import learned as lg
    if not os.path.exists(lg.WEIGHTS):
        raise SystemExit("no trained weights: run python -m flowfpmpp_gb300.train_learned --out " + lg.WEIGHTS)
    net = lg.LearnedGuess.load()
    rng = np.random.default_rng(20261)
    ax, ay, az = lg.training_grid(256, 256, 128)
    rows = []
    # the flexible CG with the network as preconditioner is slow (see the
    # design notes): only with --arms naming fcg_learned
    fcg = "fcg_learned" in args.arms.split(",")
    for s_ in range(args.warmup + args.steps):
        axis = int(rng.integers(0, 3))
        p = lg.DeviceProblem(lg.frame_for(lg.random_bodies(rng, ax, ay, az), ax, ay, az, axis))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        _, sw0, r0, _ = p.solve("pcg", tol=1e-10)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        _, sw1, r1, fb = p.solve("pcg", tol=1e-10, net=net)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        sw2, r2 = 0, 0.0
        if fcg:
            _, sw2, r2, _ = p.solve("fcg_learned", tol=1e-10, net=net)
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        # the multigrid-preconditioned refinement from phi = 0 and from the guess
        _, sw3, r3, _ = p.solve("pcg_mg", tol=1e-10)
        torch.cuda.synchronize()
        t5 = time.perf_counter()
        _, sw4, r4, fb4 = p.solve("pcg_mg", tol=1e-10, net=net)
        torch.cuda.synchronize()
        t6 = time.perf_counter()
        if s_ >= args.warmup:
            rows.append((sw0, t2 - t1, r0, sw1, t3 - t2, r1, fb, sw2, t4 - t3, r2, sw3, t5 - t4, r3, sw4, t6 - t5, r4,
                         fb4))
    a = np.array(rows, dtype=np.float64)
    line = {"metric": "FP64 PCG solve time to 1e-10 with the learned initial guess vs from phi = 0",
            "value": float(a[:, 4].mean()), "unit": "s per body", "higher_is_better": False, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "data": "synthetic (seeded random bodies)",
            "config": {"workload": "unseen bodies 256x256x128, network trained on 2000 bodies at 128x128x64",
                       "tolerance": 1e-10, "bodies": len(rows)},
            "plain": {"seconds": float(a[:, 1].mean()), "iterations": float(a[:, 0].mean())},
            "learned": {"seconds": float(a[:, 4].mean()), "iterations": float(a[:, 3].mean()),
                        "fallbacks": int(a[:, 6].sum()), "max_residual": float(a[:, 5].max())},
            "iteration_ratio": float(a[:, 0].sum() / a[:, 3].sum()),
            "time_ratio": float(a[:, 1].sum() / a[:, 4].sum()),
            "mg": {"seconds": float(a[:, 11].mean()), "iterations": float(a[:, 10].mean()),
                   "max_residual": float(a[:, 12].max())},
            "learned_mg": {"seconds": float(a[:, 14].mean()), "iterations": float(a[:, 13].mean()),
                           "fallbacks": int(a[:, 16].sum()), "max_residual": float(a[:, 15].max()),
                           "iteration_ratio_vs_mg": float(a[:, 10].sum() / a[:, 13].sum()),
                           "time_ratio_vs_mg": float(a[:, 11].sum() / a[:, 14].sum())},
            "mg_vs_plain_time_ratio": float(a[:, 1].sum() / a[:, 11].sum())}
    if fcg:
        line["fcg_learned"] = {"seconds": float(a[:, 8].mean()), "iterations": float(a[:, 7].mean()),
                               "max_residual": float(a[:, 9].max()),
                               "iteration_ratio": float(a[:, 0].sum() / a[:, 7].sum()),
                               "time_ratio": float(a[:, 1].sum() / a[:, 8].sum())}
    print(json.dumps(line), flush=True)


def run_frames(args):
    """256 uneven 2-D foil frames (96^2..512^2 cells), phi_x and
    phi_y to a 1e-10 max-norm residual and the four partition terms for both,
    all frames batched; host arrays in and out (the C ABI call a user makes)."""
    import torch
    from flowfpmpp_gb300 import build as fbuild
    fbuild.build()
    from flowfpmpp_gb300 import partition as pt
    from flowfpmpp_gb300 import workloads
    frames = workloads.foil_frames(nframes=args.frames)
    cells = sum(f["nx"] * f["ny"] for f in frames)
    for _ in range(args.warmup):
        pt.partition_frames_2d(frames, tolerance=1e-10)
    torch.cuda.synchronize()
    import flowfpmpp_gb300
    lib = flowfpmpp_gb300.lib()
    lib.fpm_timing_enable(1)
    nl, tot = ctypes.c_longlong(), ctypes.c_double()
    lib.fpm_timing_read(4, ctypes.byref(nl), ctypes.byref(tot), 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        terms, sweeps, res = pt.partition_frames_2d(frames, tolerance=1e-10)
    el = (time.perf_counter() - t0) / args.steps
    lib.fpm_timing_read(4, ctypes.byref(nl), ctypes.byref(tot), 1)
    lib.fpm_timing_enable(0)
    line = {"metric": "batched 2-D frames: phi_x, phi_y to 1e-10 and the four FPM terms",
            "value": len(frames) / el, "unit": "frames/s", "higher_is_better": True, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "seconds_per_batch": el, "data": "synthetic (seeded)",
            "config": {"workload": f"{len(frames)} foil frames 96^2..512^2, ratio 1.02", "frames": len(frames),
                       "cells_2d": int(cells), "tolerance": 1e-10},
            "cell_potentials_per_s": 2 * cells / el, "max_residual": float(np.max(res)),
            "fp32_iterations": {"max": int(sweeps.max()), "mean": float(sweeps.mean())},
            "batched_iterations": {"count": int(nl.value) // max(args.steps, 1),
                                   "ms_each": tot.value / max(nl.value, 1)},
            "all_converged": bool(np.all(res <= 1e-10))}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- C3 inside the default line
C3_FIXTURE = os.path.join(ROOT, "tests", "golden", "c3_phix_oracle.npz")
MG_LEVEL0_BYTES = 56   # multigrid level 0, per cell, right-hand side and iteration: spmv 25, residual 17.5, smoothing 13.5
FP64_PCG_BYTES = 112   # the reference's FP64 PCG iteration, per cell (14 fields)


def fixture_error(phi_padded, nx, ny, fx):
    """Relative max-norm error of phi_x at the oracle fixture's sampled cells
    (normalised by the oracle field's max |phi|) and of the whole-field sum."""
    interior = np.asarray(phi_padded).reshape((nx + 2, ny + 2, -1), order="F")[1:nx + 1, 1:ny + 1, :]
    flat = interior.ravel(order="F")
    samp = flat[::int(fx["stride"])]
    ref = fx["sample"]
    scale = float(fx["checksum"][2])
    return {"rel_linf_sampled": float(np.abs(samp - ref).max() / scale), "cells_compared": int(ref.size),
            "sum_rel": float(abs(flat.sum() - fx["checksum"][0]) / float(fx["checksum"][1]))}


def oracle_pcg_iteration_s(f, body, faces, threads):
    """Seconds per FP64 PCG iteration of the oracle on the host cores: two
    bounded solves (10 and 30 iterations from phi = 0) differenced, so the
    operator build, the true residuals and the gauge cancel."""
    import oracle as orc
    orc.build()
    orc.set_threads(threads)
    times = []
    for its in (10, 30):
        phi = f["phi"].copy(order="F")
        t0 = time.perf_counter()
        orc.solve_stairstep_poisson_3d(phi, f["rhs"], f["solid"], body, *faces, f["xc"], f["yc"], f["zc"], f["dx"],
                                       f["dy"], f["dz"], 1e-300, its, 1000000, "pcg")
        times.append(time.perf_counter() - t0)
    orc.set_threads(1)
    return (times[1] - times[0]) / 20.0


TERMS_MULTI_BYTES = 220   # nine flow fields + solid once, phi and five outputs per potential (three potentials)
TERMS_SINGLE_BYTES = 124  # one potential per call: phi, nine flow fields, solid, five outputs


def c3_densities(lib, f, phis_host, faces_host, faces_dev, bgs, dsolid, dax, stream, check_oracle):
    """Force densities of the three potentials in the C1-style flow on the C3
    grid: the one-pass kernel for all three (double-float per cell) timed
    against three calls of the bit-identical FP64 kernel; phi_x's fields and
    integrals against the oracle's FP64 densities on the same potential."""
    import torch
    from flowfpmpp_gb300 import workloads
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    n3 = nx * ny * nz
    fl = workloads.flow_c1(f)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
    dflow = [dev(fl[k]) for k in ("u", "v", "w", "ox", "oy", "oz", "ax", "ay", "az")]
    dphi = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in phis_host]
    outs = [torch.empty(n3, dtype=torch.float64, device="cuda") for _ in range(15)]
    bounds = np.array([-1e300, 1e300] * 3)
    VP = ctypes.c_void_p
    bg = np.ascontiguousarray(np.concatenate(bgs))
    tot = (ctypes.c_double * 6)()

    def fused():
        rc = lib.fpm_compute_stairstep_fpm_terms_3d_multi_dev(
            3, (VP * 3)(*[t.data_ptr() for t in dphi]), *[VP(t.data_ptr()) for t in dflow], VP(dsolid.data_ptr()),
            bg.ctypes.data_as(VP), *[VP(t.data_ptr()) for t in dax], (VP * 18)(*[t.data_ptr() for t in faces_dev]),
            bounds.ctypes.data_as(VP), (VP * 15)(*[t.data_ptr() for t in outs]), tot, nx, ny, nz,
            VP(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fpm_last_error().decode())

    def single():
        t2 = (ctypes.c_double * 2)()
        for m in range(3):
            b = np.ascontiguousarray(bgs[m])
            rc = lib.fpm_compute_stairstep_fpm_terms_3d_dev(
                VP(dphi[m].data_ptr()), *[VP(t.data_ptr()) for t in dflow], VP(dsolid.data_ptr()),
                b.ctypes.data_as(VP), *[VP(t.data_ptr()) for t in dax],
                *[VP(t.data_ptr()) for t in faces_dev[6 * m:6 * m + 6]], bounds.ctypes.data_as(VP),
                *[VP(o.data_ptr()) for o in outs[5 * m:5 * m + 5]], t2, nx, ny, nz, VP(stream.cuda_stream))
            if rc != 0:
                raise RuntimeError(lib.fpm_last_error().decode())

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps / 1e3

    t_single = timed(single, 2)
    t_fused = timed(fused, 5)
    res = {"kernel": "k_terms_multi<3>", "seconds_three_potentials": t_fused,
           "bytes_per_cell": TERMS_MULTI_BYTES, "gbs": TERMS_MULTI_BYTES * float(n3) / t_fused / 1e9,
           "arithmetic": "double-float per cell (48-bit significand), FP64 storage and integrals",
           "integrals": [tot[m] for m in range(6)],
           "single_potential_fp64_kernel": {"kernel": "k_terms", "seconds_three_calls": t_single,
                                            "gbs": 3 * TERMS_SINGLE_BYTES * float(n3) / t_single / 1e9,
                                            "arithmetic": "f64, bit-identical to the oracle"},
           "speedup_vs_three_calls": t_single / t_fused}
    if check_oracle:
        import oracle as orc
        ro = orc.compute_stairstep_fpm_terms_3d(phis_host[0].reshape(f["phi"].shape, order="F"), fl["u"], fl["v"],
                                                fl["w"], fl["ox"], fl["oy"], fl["oz"], fl["ax"], fl["ay"], fl["az"],
                                                f["solid"], bgs[0], f["xc"], f["yc"], f["zc"], f["dx"], f["dy"],
                                                f["dz"], *faces_host[0], bounds)
        fused()
        torch.cuda.synchronize()
        errs = [rel_linf(outs[c].cpu().numpy(), np.asarray(ro[c]).ravel(order="F")) for c in range(5)]
        scale = max(abs(ro[5][0]), abs(ro[5][1]), 1e-300)
        res["phi_x_vs_oracle"] = {"fields_rel_linf": max(errs), "per_field": errs,
                                  "integrals_rel": max(abs(tot[0] - ro[5][0]), abs(tot[1] - ro[5][1])) / scale,
                                  "tolerance": 1e-8}
    return res


def pcg_c3(args, lib):
    """The PCG half of the metric on the three-ellipsoid 384x384x192 grid:
    phi_x, phi_y, phi_z to a 1e-10 max-norm residual with the multigrid-
    preconditioned FP32 PCG in FP64 refinement (all three per launch, timed
    over solves) and with plain FP64 PCG (one solve of the three), phi_x of
    both against the oracle's FP64 PCG fixture, and the oracle's per-iteration
    time on the host cores times the FP64 iteration count as the CPU figure."""
    import torch
    from flowfpmpp_gb300 import stairstep as ss
    from flowfpmpp_gb300 import workloads
    f = workloads.ellipsoids_grid()
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    n3 = nx * ny * nz
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
    faces_host, faces_dev, bgs, rhss = [], [], [], []
    for axis in range(3):
        body = np.zeros(3)
        body[axis] = 1.0
        faces = [x.copy(order="F") for x in f["faces"]]
        ss.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], body, *faces, f["dx"], f["dy"], f["dz"])
        faces_host.append(faces)
        faces_dev += [dev(x) for x in faces]
        bgs.append(body)
        rhss.append(dev(f["rhs"]))
    phis = [dev(f["phi"]) for _ in range(3)]
    dsolid = dev(f["solid"])
    dax = [dev(f[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    VP = ctypes.c_void_p
    bg = np.ascontiguousarray(np.concatenate(bgs))
    stream = torch.cuda.current_stream()

    def solve(method):
        for t in phis:
            t.zero_()
        sweeps = (ctypes.c_int * 3)()
        res = (ctypes.c_double * 3)()
        rc = lib.fpm_solve_stairstep_multi_dev(
            3, (VP * 3)(*[t.data_ptr() for t in phis]), (VP * 3)(*[t.data_ptr() for t in rhss]), VP(dsolid.data_ptr()),
            bg.ctypes.data_as(VP), (VP * 18)(*[t.data_ptr() for t in faces_dev]), *[VP(t.data_ptr()) for t in dax],
            nx, ny, nz, ctypes.c_double(1e-10), 2000000, 50, method, sweeps, res, VP(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fpm_last_error().decode())
        return list(sweeps), list(res)

    def timer(which):
        nl, tot = ctypes.c_longlong(), ctypes.c_double()
        lib.fpm_timing_read(which, ctypes.byref(nl), ctypes.byref(tot), 1)
        return nl.value, tot.value

    out = {}
    for label, method, warm, steps in (("mg", 4, 1, 2), ("fp64", 0, 0, 1)):
        for _ in range(warm):
            solve(method)
        torch.cuda.synchronize()
        lib.fpm_timing_enable(1)
        timer(3), timer(2)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            sw, res = solve(method)
        e1.record(stream)
        torch.cuda.synchronize()
        lib.fpm_timing_enable(0)
        it_mixed, it_fp64 = timer(3), timer(2)
        out[label] = {"seconds": e0.elapsed_time(e1) / steps / 1e3, "iterations": sw, "residual": res,
                      "solves_timed": steps, "phi": [t.cpu().numpy().copy() for t in phis],
                      "iter_timer": {"mg": it_mixed, "fp64": it_fp64}}
    line = {"workload": "3 ellipsoids 384x384x192, ratio 1.02, phi_x/phi_y/phi_z to 1e-10 max-norm residual",
            "grid": [nx, ny, nz], "tolerance": 1e-10, "check_interval": 50,
            "value": out["mg"]["seconds"], "unit": "s", "higher_is_better": False,
            "arm": "FP32 PCG with an aggregation-multigrid preconditioner in FP64 refinement (all three per launch)",
            "speedup_vs_fp64": out["fp64"]["seconds"] / out["mg"]["seconds"]}
    fx = None
    if os.path.exists(C3_FIXTURE):
        fx = np.load(C3_FIXTURE)
        if tuple(int(x) for x in fx["grid"]) != (nx, ny, nz):
            fx = None
    for label in ("mg", "fp64"):
        o = out[label]
        d = {k: o[k] for k in ("seconds", "iterations", "residual", "solves_timed")}
        if fx is not None:
            d["phi_x_vs_oracle"] = fixture_error(o["phi"][0], nx, ny, fx)
        line[label] = d
    line["fp64"]["iterations_oracle_phi_x"] = int(fx["iterations"]) if fx is not None else None
    line["mg"]["vs_gpu_fp64_rel_linf"] = [rel_linf(a, b) for a, b in zip(out["mg"]["phi"], out["fp64"]["phi"])]
    # roofline of the iteration: algorithmic bytes of level 0 (coarse levels
    # not counted) and of the reference's FP64 iteration over their timers
    nl, ms = out["mg"]["iter_timer"]["mg"]
    mg_bytes = MG_LEVEL0_BYTES * float(n3) * sum(out["mg"]["iterations"]) * out["mg"]["solves_timed"]
    nl64, ms64 = out["fp64"]["iter_timer"]["fp64"]
    fp64_bytes = FP64_PCG_BYTES * float(n3) * sum(out["fp64"]["iterations"])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    line["roofline"] = {
        "bound": "hbm", "unit": "GB/s", "peak": peak,
        "mg_iteration": {"achieved": mg_bytes / (ms / 1e3) / 1e9, "frac": mg_bytes / (ms / 1e3) / 1e9 / peak,
                         "bytes_per_cell_rhs": MG_LEVEL0_BYTES, "iteration_ms_all_rhs": ms / max(nl, 1),
                         "note": "level-0 bytes over the whole iteration time (coarse levels included in the time)"},
        "fp64_iteration": {"achieved": fp64_bytes / (ms64 / 1e3) / 1e9,
                           "frac": fp64_bytes / (ms64 / 1e3) / 1e9 / peak, "bytes_per_cell": FP64_PCG_BYTES,
                           "iteration_ms": ms64 / max(nl64, 1)}}
    if not args.no_densities:
        line["densities"] = c3_densities(lib, f, out["mg"]["phi"], faces_host, faces_dev, bgs, dsolid, dax, stream,
                                         check_oracle=not args.no_cpu_baseline)
    if not args.no_cpu_baseline:
        import oracle as orc
        cores = orc.max_threads()
        per_it = oracle_pcg_iteration_s(f, bgs[0], faces_host[0], cores)
        total_its = sum(out["fp64"]["iterations"])
        line["cpu_baseline"] = {"value": per_it * total_its, "unit": "s", "cores": cores, "kind": "port",
                                "sample": f"oracle FP64 PCG, 20 iterations of phi_x timed ({per_it * 1e3:.1f} ms per "
                                          f"iteration, OpenMP over z-planes) x {total_its} iterations (the FP64 arm's "
                                          f"count for the three potentials)"}
    return line


# ---------------------------------------------------------------- C1 and C4 inside the default line
def multi_solve(lib, f, method, steps, warmup):
    """phi_x, phi_y, phi_z of grid f to 1e-10 through fpm_solve_stairstep_multi_dev
    (device arrays): (seconds per solve, iterations, residuals, potentials)."""
    import torch
    from flowfpmpp_gb300 import stairstep as ss
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
    faces_dev, bgs = [], []
    for axis in range(3):
        body = np.zeros(3)
        body[axis] = 1.0
        faces = [x.copy(order="F") for x in f["faces"]]
        ss.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], body, *faces, f["dx"], f["dy"], f["dz"])
        faces_dev += [dev(x) for x in faces]
        bgs.append(body)
    rhss = [dev(f["rhs"]) for _ in range(3)]
    phis = [dev(f["phi"]) for _ in range(3)]
    dsolid = dev(f["solid"])
    dax = [dev(f[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    VP = ctypes.c_void_p
    bg = np.ascontiguousarray(np.concatenate(bgs))
    stream = torch.cuda.current_stream()
    sweeps = (ctypes.c_int * 3)()
    res = (ctypes.c_double * 3)()

    def solve():
        for t in phis:
            t.zero_()
        rc = lib.fpm_solve_stairstep_multi_dev(
            3, (VP * 3)(*[t.data_ptr() for t in phis]), (VP * 3)(*[t.data_ptr() for t in rhss]), VP(dsolid.data_ptr()),
            bg.ctypes.data_as(VP), (VP * 18)(*[t.data_ptr() for t in faces_dev]), *[VP(t.data_ptr()) for t in dax],
            nx, ny, nz, ctypes.c_double(1e-10), 2000000, 50, method, sweeps, res, VP(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fpm_last_error().decode())

    for _ in range(warmup):
        solve()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        solve()
    e1.record(stream)
    torch.cuda.synchronize()
    shape = f["phi"].shape
    return (e0.elapsed_time(e1) / steps / 1e3, list(sweeps), list(res),
            [t.cpu().numpy().reshape(shape, order="F") for t in phis])


def pcg_c1(args, lib):
    """The C1 case: sphere r = 0.5 on the 64x64x32 grid of ratio 1.03,
    phi_x, phi_y, phi_z to 1e-10 with plain FP64 PCG and with the multigrid
    refinement, each potential against the oracle's FP64 PCG (1e-9), and the
    oracle's whole three-potential solve on the host cores."""
    from flowfpmpp_gb300 import workloads
    import oracle as orc
    f = workloads.sphere_grid()
    out = {}
    for label, method in (("fp64", 0), ("mg", 4)):
        sec, sw, res, phis = multi_solve(lib, f, method, steps=5, warmup=2)
        out[label] = {"seconds": sec, "iterations": sw, "residual": res, "phi": phis}
    orc.build()
    cores = orc.max_threads()
    orc.set_threads(cores)
    ref, t0 = [], time.perf_counter()
    for axis in range(3):
        body = np.zeros(3)
        body[axis] = 1.0
        faces = [x.copy(order="F") for x in f["faces"]]
        orc.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], body, *faces, f["dx"], f["dy"], f["dz"])
        phi = f["phi"].copy(order="F")
        orc.solve_stairstep_poisson_3d(phi, f["rhs"], f["solid"], body, *faces, f["xc"], f["yc"], f["zc"], f["dx"],
                                       f["dy"], f["dz"], 1e-10, 2000000, 50, "pcg")
        ref.append(phi)
    el = time.perf_counter() - t0
    orc.set_threads(1)
    line = {"workload": "sphere r=0.5, 64x64x32 on [-4,4]^2 x [-2,2], ratio 1.03, phi_x/phi_y/phi_z to 1e-10",
            "value": out["mg"]["seconds"], "unit": "s", "higher_is_better": False,
            "speedup_vs_fp64": out["fp64"]["seconds"] / out["mg"]["seconds"],
            "cpu_baseline": {"value": el, "unit": "s", "cores": cores, "kind": "port",
                             "sample": "the oracle's FP64 PCG of the three potentials (OpenMP over z-planes)"}}
    for label in ("fp64", "mg"):
        o = out[label]
        line[label] = {"seconds": o["seconds"], "iterations": o["iterations"], "residual": o["residual"],
                       "rel_linf_vs_oracle": [rel_linf(a, b) for a, b in zip(o["phi"], ref)]}
    line["parity_pass"] = all(x <= 1e-9 for lb in ("fp64", "mg") for x in line[lb]["rel_linf_vs_oracle"])
    return line


def oracle_frame(fr):
    """The reference foil example's per-frame work (examples/flapping_foil_fpm.f90:61-81)
    on the oracle: phi_x, phi_y by FP64 PCG to 1e-10, then fpm_partition_terms_2d."""
    import oracle as orc
    from flowfpmpp_gb300.workloads import frame_as_stairstep
    s = frame_as_stairstep(fr)
    terms, phis = np.zeros((2, 4)), []
    for d in range(2):
        body = np.zeros(3)
        body[d] = 1.0
        faces = [x.copy(order="F") for x in s["faces"]]
        orc.enforce_stairstep_compatibility_3d(s["rhs"], s["solid"], body, *faces, s["dx"], s["dy"], s["dz"])
        phi = s["phi"].copy(order="F")
        orc.solve_stairstep_poisson_3d(phi, s["rhs"], s["solid"], body, *faces, s["xc"], s["yc"], s["zc"], s["dx"],
                                       s["dy"], s["dz"], 1e-10, 2000000, 50, "pcg")
        p2 = np.asfortranarray(phi[1:fr["nx"] + 1, 1:fr["ny"] + 1, 0])
        terms[d], _, _ = orc.fpm_partition_terms_2d(p2, body[:2], fr["u"], fr["v"], fr["solid"], fr["xf"], fr["yf"],
                                                    fr["kin"], fr["ring"], fr["dt"], fr["nu"])
        phis.append(p2)
    return terms, phis


def frames_c4(args, lib):
    """The C4 batch: 256 uneven 2-D foil frames (96^2..512^2, ratio 1.02),
    phi_x and phi_y to 1e-10 and the four partition terms each, host arrays in
    and out through fpm_partition_frames_2d; the three smallest frames against
    the oracle, and the oracle's time on them scaled to the batch's cells."""
    import torch
    from flowfpmpp_gb300 import partition as pt
    from flowfpmpp_gb300 import workloads
    import oracle as orc
    frames = workloads.foil_frames()
    cells = sum(f["nx"] * f["ny"] for f in frames)
    pt.partition_frames_2d(frames, tolerance=1e-10)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pt.partition_frames_2d(frames, tolerance=1e-10)
    el = time.perf_counter() - t0
    # the same call again with the potentials downloaded, for the oracle check
    t0 = time.perf_counter()
    terms, sweeps, res, phis = pt.partition_frames_2d(frames, tolerance=1e-10, return_phi=True)
    el_phi = time.perf_counter() - t0
    orc.build()
    cores = orc.max_threads()
    orc.set_threads(cores)
    pick = sorted(range(len(frames)), key=lambda m: frames[m]["nx"] * frames[m]["ny"])[:3]
    errs_phi, errs_terms, t_orc, cells_orc = [], [], 0.0, 0
    for m in pick:
        t1 = time.perf_counter()
        ot, op = oracle_frame(frames[m])
        t_orc += time.perf_counter() - t1
        cells_orc += frames[m]["nx"] * frames[m]["ny"]
        for d in range(2):
            errs_phi.append(rel_linf(phis[m][d], op[d]))
        errs_terms.append(float(np.abs(terms[m] - ot).max() / max(np.abs(ot).max(), 1e-300)))
    orc.set_threads(1)
    cpu_s = t_orc * cells / cells_orc
    return {"workload": "256 foil frames 96^2..512^2, ratio 1.02, phi_x/phi_y to 1e-10 + 4 terms each",
            "value": len(frames) / el, "unit": "frames/s", "higher_is_better": True, "seconds_per_batch": el,
            "seconds_per_batch_with_potentials_out": el_phi,
            "cells_2d": int(cells), "max_residual": float(np.max(res)), "all_converged": bool(np.all(res <= 1e-10)),
            "iterations": {"max": int(sweeps.max()), "mean": float(sweeps.mean())},
            "path": "all frames' pairs in the same launches (batched 2-D multigrid-preconditioned FP32 PCG in FP64 "
                    "refinement) until 80 % of the pairs have converged, the rest each by its own multigrid call",
            "vs_oracle": {"frames": pick, "phi_rel_linf": max(errs_phi), "terms_rel": max(errs_terms),
                          "tolerance": {"phi": 1e-9, "terms": 1e-8}},
            "cpu_baseline": {"value": len(frames) / cpu_s, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": f"oracle FP64 PCG + terms of the 3 smallest frames in {t_orc:.1f} s, scaled "
                                       f"by cells to the batch"}}


# ---------------------------------------------------------------- force densities alone
def run_densities(args):
    """fpm_compute_stairstep_fpm_terms_3d_multi_dev for three seeded random
    potentials and flow fields on the three-ellipsoid grid (default
    384x384x192; --grid for a smaller one), timed over `steps` calls."""
    import torch
    from flowfpmpp_gb300 import build as fbuild
    fbuild.build()
    import flowfpmpp_gb300
    from flowfpmpp_gb300 import workloads
    lib = flowfpmpp_gb300.lib()
    f = workloads.ellipsoids_grid(*args.grid) if args.grid else workloads.ellipsoids_grid()
    nx, ny, nz = f["nx"], f["ny"], f["nz"]
    n3 = nx * ny * nz
    g = torch.Generator(device="cuda").manual_seed(5)
    phis = [torch.randn((nx + 2) * (ny + 2) * nz, dtype=torch.float64, device="cuda", generator=g) for _ in range(3)]
    flow = [torch.randn(n3, dtype=torch.float64, device="cuda", generator=g) for _ in range(9)]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
    dsolid = dev(f["solid"])
    dax = [dev(f[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    faces = [dev(x) for _ in range(3) for x in f["faces"]]
    outs = [torch.empty(n3, dtype=torch.float64, device="cuda") for _ in range(15)]
    bounds = np.array([-1e300, 1e300] * 3)
    bg = np.array([1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0])
    VP = ctypes.c_void_p
    tot = (ctypes.c_double * 6)()
    stream = torch.cuda.current_stream()

    def call():
        rc = lib.fpm_compute_stairstep_fpm_terms_3d_multi_dev(
            3, (VP * 3)(*[t.data_ptr() for t in phis]), *[VP(t.data_ptr()) for t in flow], VP(dsolid.data_ptr()),
            bg.ctypes.data_as(VP), *[VP(t.data_ptr()) for t in dax], (VP * 18)(*[t.data_ptr() for t in faces]),
            bounds.ctypes.data_as(VP), (VP * 15)(*[t.data_ptr() for t in outs]), tot, nx, ny, nz,
            VP(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fpm_last_error().decode())

    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / max(args.steps, 1) / 1e3
    print(json.dumps({"metric": "force densities of three potentials in one pass", "value": sec, "unit": "s",
                      "higher_is_better": False, "steps": args.steps, "warmup": args.warmup,
                      "config": {"workload": f"random fields on the three-ellipsoid grid {nx}x{ny}x{nz}",
                                 "grid": [nx, ny, nz]},
                      "gbs": 220.0 * n3 / sec / 1e9, "bytes_per_cell": 220}), flush=True)


# ---------------------------------------------------------------- GPU arm
# Sweep kernels of the Jacobi methods: (C ABI method id, timer id, kernel,
# arithmetic, FP64 instructions per cell or None).
JACOBI_METHODS = {
    "jacobi_fma": (6, 1, "k_jacobi_f64_fma", "f64 (fused multiply-add)", 8),
    "jacobi_tf": (7, 5, "k_jacobi_tf_tma", "f64 storage, triple-float arithmetic (about 2^-60 before the FP64 "
                                           "rounding)", None),
    "jacobi": (1, 1, "k_jacobi_f64", "f64 (separately rounded, bit-identical to the oracle per sweep)", 15),
    "jacobi_df": (2, 0, "k_jacobi_df_tma", "f32x2 double-float (48-bit significand)", None),
}


def oracle_solve(f, faces, threads):
    """The oracle's 2000-sweep weighted-Jacobi solve of the same problem on
    `threads` host cores (operator build, sweeps, residual check, gauge):
    returns (phi, seconds)."""
    import oracle as orc
    orc.build()
    orc.set_threads(threads)
    phi = f["phi"].copy(order="F")
    t0 = time.perf_counter()
    sw, _ = orc.solve_stairstep_poisson_3d(phi, f["rhs"], f["solid"], f["body"], *faces, f["xc"], f["yc"], f["zc"],
                                           f["dx"], f["dy"], f["dz"], -1.0, SWEEPS, SWEEPS, "jacobi")
    el = time.perf_counter() - t0
    orc.set_threads(1)
    assert sw == SWEEPS
    return phi, el


def rel_linf(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    import torch
    torch.cuda.set_device(local)
    if args.workload == "learned_guess":
        if rank == 0:
            run_learned(args)
        return
    if args.workload == "densities":
        if rank == 0:
            run_densities(args)
        return
    if args.workload != "jacobi256":
        if rank == 0:
            run_frames(args) if args.workload == "foil_frames" else run_pcg(args)
        return
    from flowfpmpp_gb300.replicas import Replicas
    reps = Replicas(world=world, rank=rank)  # replicas only: no collective on the data path
    barrier, max_over_ranks = reps.barrier, reps.max

    from flowfpmpp_gb300 import build as fbuild
    fbuild.build()
    import flowfpmpp_gb300
    from flowfpmpp_gb300 import stairstep as ss
    lib = flowfpmpp_gb300.lib()
    lib.fpm_kernel_launches.restype = ctypes.c_longlong

    n = args.n
    head = args.method
    f = workload(n)
    faces = [a.copy(order="F") for a in f["faces"]]
    ss.enforce_stairstep_compatibility_3d(f["rhs"], f["solid"], f["body"], *faces, f["dx"], f["dy"], f["dz"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).cuda()
    d_phi = dev(f["phi"])
    d_rhs, d_solid = dev(f["rhs"]), dev(f["solid"])
    d_faces = [dev(a) for a in faces]
    d_axes = [dev(f[k]) for k in ("xc", "yc", "zc", "dx", "dy", "dz")]
    bg = np.ascontiguousarray(f["body"])
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    sw, res = ctypes.c_int(), ctypes.c_double()
    stream = torch.cuda.current_stream()

    def step(method):
        d_phi.zero_()
        rc = lib.fpm_solve_stairstep_poisson_3d_dev(
            P(d_phi), P(d_rhs), P(d_solid), bg.ctypes.data_as(ctypes.c_void_p), *[P(t) for t in d_faces],
            *[P(t) for t in d_axes], n, n, n, ctypes.c_double(-1.0), SWEEPS, SWEEPS, JACOBI_METHODS[method][0],
            ctypes.byref(sw), ctypes.byref(res), ctypes.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fpm_last_error().decode())

    def sweep_ms(method):
        nl, tot = ctypes.c_longlong(), ctypes.c_double()
        lib.fpm_timing_read(JACOBI_METHODS[method][1], ctypes.byref(nl), ctypes.byref(tot), 1)
        return tot.value / max(nl.value, 1)

    def timed(method, steps, warmup, clocks=False):
        """(ms per solve, ms per sweep kernel, kernel launches, clock summary)"""
        for _ in range(warmup):
            step(method)
        assert sw.value == SWEEPS
        barrier()
        torch.cuda.synchronize()
        lib.fpm_timing_enable(1)
        sweep_ms(method)  # clears the counter
        launches0 = lib.fpm_kernel_launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clk = ClockSampler(local) if clocks else None
        if clk:
            clk.__enter__()
        e0.record(stream)
        for _ in range(steps):
            step(method)
        e1.record(stream)
        torch.cuda.synchronize()
        if clk:
            clk.__exit__(None, None, None)
        launches = lib.fpm_kernel_launches() - launches0
        lib.fpm_timing_enable(0)
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1) / steps)
        return ms, sweep_ms(method), launches, (clk.summary() if clk else None)

    ms, head_sweep_ms, launches, clocks = timed(head, args.steps, args.warmup, clocks=True)
    value = world * algorithmic_gb(n) / (ms / 1e3)
    residual = res.value
    phis = {head: d_phi.cpu().numpy().reshape(f["phi"].shape, order="F").copy()}
    others = {}
    if not args.head_only:
        for m in JACOBI_METHODS:
            if m == head:
                continue
            oms, osw, _, _ = timed(m, 2, 1)
            phis[m] = d_phi.cpu().numpy().reshape(f["phi"].shape, order="F").copy()
            others[m] = {"dtype": JACOBI_METHODS[m][3], "kernel": JACOBI_METHODS[m][2],
                         "value": world * algorithmic_gb(n) / (oms / 1e3), "unit": "GB/s", "ms_per_solve": oms,
                         "sweep_us": osw * 1e3,
                         "sweep_gbs": BYTES_PER_CELL_SWEEP * float(n) ** 3 / (osw / 1e3) / 1e9}

    # e2e through the host-array C ABI with pinned buffers
    def pinned(a):
        a = np.asarray(a)
        ptr = lib.fpm_host_alloc(a.nbytes)
        buf = (ctypes.c_char * a.nbytes).from_address(ptr)
        out = np.frombuffer(buf, dtype=a.dtype).reshape(a.shape, order="F")
        out[...] = a
        return out, ptr

    h_phi, p0 = pinned(f["phi"])
    h_in = [pinned(x) for x in [f["rhs"], f["solid"], *faces, f["xc"], f["yc"], f["zc"], f["dx"], f["dy"], f["dz"]]]
    h2d = h_phi.nbytes + sum(x[0].nbytes for x in h_in)
    d2h = h_phi.nbytes

    def e2e_step():
        h_phi[...] = 0.0
        args_ = [h_phi.ctypes.data_as(ctypes.c_void_p), h_in[0][0].ctypes.data_as(ctypes.c_void_p),
                 h_in[1][0].ctypes.data_as(ctypes.c_void_p), bg.ctypes.data_as(ctypes.c_void_p)]
        args_ += [x[0].ctypes.data_as(ctypes.c_void_p) for x in h_in[2:]]
        rc = lib.fpm_solve_stairstep_poisson_3d(*args_, n, n, n, ctypes.c_double(-1.0), SWEEPS, SWEEPS,
                                                JACOBI_METHODS[head][0], ctypes.byref(sw), ctypes.byref(res))
        if rc != 0:
            raise RuntimeError(lib.fpm_last_error().decode())

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    e2e_steps = max(1, args.steps // 2)
    for _ in range(e2e_steps):
        e2e_step()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) / e2e_steps * 1e3)
    e2e_value = world * algorithmic_gb(n) / (e2e_ms / 1e3)
    e2e_parity = rel_linf(h_phi, phis[head])
    for x in [p0] + [x[1] for x in h_in]:
        lib.fpm_host_free(ctypes.c_void_p(x))

    fp64_rate = ctypes.c_double()
    if lib.fpm_measure_fp64_rate(ctypes.byref(fp64_rate), ctypes.c_void_p(stream.cuda_stream)) != 0:
        raise RuntimeError(lib.fpm_last_error().decode())

    pcg = c1 = c4 = None
    if not args.no_pcg and world == 1:
        pcg = pcg_c3(args, lib)
        c1 = pcg_c1(args, lib)
        c4 = frames_c4(args, lib)

    reps.close()
    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    achieved = BYTES_PER_CELL_SWEEP * float(n) ** 3 / (head_sweep_ms / 1e3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", f"{JACOBI_METHODS[head][2]}_256cubed.json")
    if n == 256 and os.path.exists(prof):
        try:
            traffic = json.load(open(prof)).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            traffic = None
    roofline = {"bound": "hbm", "kernel": JACOBI_METHODS[head][2], "achieved": achieved, "peak": peak,
                "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "avg_launch_us": head_sweep_ms * 1e3, "algorithmic_bytes_per_launch": BYTES_PER_CELL_SWEEP * n ** 3}
    fp64_per_cell = JACOBI_METHODS[head][4]
    if fp64_per_cell:
        got = fp64_per_cell * float(n) ** 3 / (head_sweep_ms / 1e3)
        roofline["fp64_pipe"] = {"instructions_per_cell": fp64_per_cell, "achieved_per_s": got,
                                 "peak_per_s": fp64_rate.value, "frac": got / fp64_rate.value,
                                 "peak_source": "measured in this run (fpm_measure_fp64_rate)"}
    for m, o in others.items():
        o["hbm_frac"] = o["sweep_gbs"] / peak
        if JACOBI_METHODS[m][4]:
            o["fp64_pipe_frac"] = JACOBI_METHODS[m][4] * float(n) ** 3 / (o["sweep_us"] * 1e-6) / fp64_rate.value
    if "jacobi_df" in others:
        traffic_df = None
        prof = os.path.join(ROOT, "profiles", "jacobi_df_256cubed.json")
        if n == 256 and os.path.exists(prof):
            traffic_df = json.load(open(prof)).get("dram_bytes_per_launch")
        others["jacobi_df"]["traffic"] = traffic_df
    cpu, parity = None, None
    if world == 1 and not args.no_cpu_baseline:
        import oracle as orc
        orc.build()
        cores = orc.max_threads()
        ref_phi, el = oracle_solve(f, faces, cores)
        gbs = algorithmic_gb(n) / el
        cpu = {"value": gbs, "unit": "GB/s", "cores": cores, "kind": "port",
               "sample": f"the whole {SWEEPS}-sweep {n}^3 solve in {el:.1f} s (oracle, OpenMP over z-planes)"}
        # the reference's serial order on one core, beside the all-cores figure
        g1, _, n1, e1 = cpu_sample(n, budget_s=4.0, threads=1)
        cpu["single_core"] = {"value": g1, "unit": "GB/s", "cores": 1,
                              "sample": f"{n1} sweeps of the same operator in {e1:.1f} s (oracle, one thread)"}
        parity = {"vs": f"oracle weighted Jacobi, {SWEEPS} sweeps of the same operator, gauge removed",
                  "tolerance": 1e-12, "rel_linf": rel_linf(phis[head], ref_phi), "e2e_vs_device": e2e_parity}
        for m in others:
            others[m]["rel_linf_vs_oracle"] = rel_linf(phis[m], ref_phi)
        parity["pass"] = parity["rel_linf"] <= 1e-12
    cfg = config(n, head)
    cfg["parallelism"] = f"replicas x{world}"
    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if head in ("jacobi_fma", "jacobi", "jacobi_tf") else "f32x2",
            "arithmetic": JACOBI_METHODS[head][3], "data": "synthetic (seeded boxes)", "config": cfg,
            "roofline": roofline, "cpu_baseline": cpu, "parity": parity,
            "e2e": {"value": e2e_value, "unit": "GB/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_ms},
            "gpu_launches": int(launches), "clocks": clocks, "final_residual": residual, "other_methods": others}
    if pcg is not None:
        line["pcg_c3"] = pcg
        line["pcg_c1"] = c1
        line["frames_c4"] = c4
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
