#!/usr/bin/env python3
"""Benchmark of the staggered M^+M solve on one GB300.

Workload: solve (M^+M) x = b with M^+M = m^2 - D_eo D_oe on a 32^4 lattice,
m = 0.01, to an FP64 true residual sqrt(|b - M^+M x|^2/|b|^2) <= 1e-10 -- the
configuration the headline metric is quoted on.  Links: a thermalised
configuration of the tree-level Symanzik gauge action at beta = 3.75, made
before the timed region by the library's pure-gauge HMC from a cold start
(200 trajectories of the reference's integrator, 18 steps x 4 gauge
substeps, FP32 molecular dynamics, the first 20 without the Metropolis test
as the reference's thermalisation trajectories), then smeared by 2 stout
steps of rho = 0.15; staggered phases with antiperiodic time boundary; a
Gaussian source on the even sites.  --links-source synthetic uses seeded
U = exp(i*0.3*H) links instead (H Gaussian traceless Hermitian per link).

A step is one complete solve.  `value` is solves per second over all GPUs
(independent replicas, one per rank, weak scaling), timed with CUDA events on
the solver's stream with all inputs resident in HBM; `e2e` is the same solve
through the reference-facing C entry points with pinned host buffers, the
host->device copies of links (the two stored rows the kernels read),
phases, source and guess and the device->host copy of the solution inside
the timed region.  The plain FP64 CG
(ker_invert_openacc) is timed beside it.

--impl reference times the reference's CPU implementation of the same solve
(its FP64 CG, restated as the oracle port and run with all host threads) on
rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
PROFILE_TRAFFIC = ROOT / "profiles" / "traffic.json"
FALLBACK_HBM = 6800.0

# algorithmic bytes per output site of one hop application
# D_oe of the mixed solver per output site: links (2 rows FP32) + sign bytes + in + out
BYTES_F32_SIGN = 8 * 12 * 4 + 8 * 1 + 3 * 8 + 3 * 8      # = 440
# D_eo + M^+M epilogue + <p,s> per output site: links + sign bytes + t and p in + s out
BYTES_F32_DEO = 8 * 12 * 4 + 8 * 1 + 2 * 3 * 8 + 3 * 8        # = 464
# the same with the links in 16-bit fixed point (12 x 2 bytes per link)
BYTES_Q16_SIGN = 8 * 12 * 2 + 8 * 1 + 3 * 8 + 3 * 8      # = 248
BYTES_Q16_DEO = 8 * 12 * 2 + 8 * 1 + 2 * 3 * 8 + 3 * 8        # = 272
BYTES_F64_ANGLE = 8 * 12 * 8 + 8 * 8 + 3 * 16 + 3 * 16   # links(2 rows) + angles + in + out = 928


def run_multishift(api, L, lat, u, ph, b, dims, rank, stream, args):
    import torch
    from openstaple_gb300 import fields as F
    apx = json.loads((ROOT / "tests" / "golden" / "ratapprox.json").read_text())["order19"]
    mx = 64.0 * 1.05
    eps = mx ** (apx["exponent_num"] / apx["exponent_den"])
    ra = api.make_approx(apx["a0"] * eps, np.array(apx["a"]) * mx * eps, np.array(apx["b"]) * mx)
    order = ra.approx_order
    bm = np.stack([b] + [F.gaussian_vec3(dims, args.seed + 17 * rank + 200 + k) for k in range(3)])
    xm = lat.vec3(4 * order)
    lat.present(bm)
    lat.present(xm)

    def timed(f):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        r = f()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), r

    runs = [timed(lambda: api.multishift_batch(u, ph, args.mass, ra, bm, xm, args.res, 100000, args.delta))
            for _ in range(2)]
    ms, info = min(runs, key=lambda t: t[0])
    lat.update_host(xm)
    # the reference algorithm in FP64 on the GPU, one source after the other
    work = [lat.vec3() for _ in range(4)]
    sf, xo = lat.vec3(order), lat.vec3(order)
    for a in work + [sf, xo]:
        lat.present(a, copy=False)
    fp = api.make_ferm_param(args.mass, ph)
    fp64_ms, fp64_iters, err = 0.0, [], 0.0
    for k in range(4):
        bk = np.ascontiguousarray(bm[k])
        lat.present(bk)
        t, (st, n) = timed(lambda: api.multishift_invert(u, fp, ra, xo, bk, args.res, *work, sf, 100000))
        fp64_ms += t
        fp64_iters.append(int(n))
        lat.update_host(xo)
        err = max(err, max(rel_diff(xm[k * order + j], xo[j]) for j in range(order)))
        lat.release(bk)
    for a in work + [sf, xo, bm, xm]:
        lat.release(a)
    return {"sources": 4, "shifts": int(order), "ms": ms, "status": int(info["status"]),
            "true_residual_max": float(info["true_res"].max()), "cgm_iterations": [int(i) for i in info["iters_cgm"]],
            "fp64_multishift_invert_ms": fp64_ms, "fp64_iterations": fp64_iters, "err_vs_fp64": err,
            "speedup_vs_fp64_multishift_invert": fp64_ms / ms if ms else None}


def rel_diff(x, ref):
    """|x - ref| / |ref| over all components: the relative error of a solution
    against the FP64 solution of the same system."""
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dims", default="32,32,32,32")
    ap.add_argument("--mass", type=float, default=0.01)
    ap.add_argument("--eps", type=float, default=0.3)
    ap.add_argument("--res", type=float, default=1e-10)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true", help="skip the plain FP64 CG arm (profiling runs)")
    ap.add_argument("--solver", default="mixed", choices=["mixed", "learned"],
                    help="learned: flexible CG preconditioned by the network, trained before the timed region "
                         "on solver-produced pairs")
    ap.add_argument("--train-epochs", type=int, default=150)
    ap.add_argument("--pairs", type=int, default=8,
                    help="training pairs of the learned preconditioner (solved by the batched solver, 8 at a time)")
    ap.add_argument("--pair-res", type=float, default=None,
                    help="FP64 true residual of the training solutions (default: --res)")
    ap.add_argument("--rhs", type=int, default=1,
                    help="right-hand sides per step; >1 solves them together with the batched solver")
    ap.add_argument("--links", choices=("q16", "f32"), default="q16",
                    help="sloppy link format of the FP32 iteration (16-bit fixed point or FP32 rows)")
    ap.add_argument("--every", type=int, default=0,
                    help="reliable update every N iterations of the single-system solver (0: the delta criterion)")
    ap.add_argument("--no-multishift", action="store_true",
                    help="skip the 4-source x 19-shift multi-shift measurement reported beside the headline")
    ap.add_argument("--delta", type=float, default=1e-4,
                    help="reliable update when |r|^2 < delta * max|r|^2 since the last one")
    ap.add_argument("--links-source", choices=("thermalized", "synthetic"), default="thermalized",
                    help="thermalized: pure-gauge HMC configuration + stout smearing; synthetic: exp(i eps H) links")
    ap.add_argument("--beta", type=float, default=3.75)
    ap.add_argument("--therm", type=int, default=200, help="pure-gauge HMC trajectories from the cold start")
    ap.add_argument("--therm-nometro", type=int, default=20,
                    help="of which the first ones skip the Metropolis test (the reference's ThermNtraj)")
    ap.add_argument("--stout", type=int, default=2, help="stout steps of rho = 0.15 on the thermalised links")
    ap.add_argument("--no-link-cache", action="store_true",
                    help="always generate the thermalised configuration (no ILDG cache file is read or written)")
    return ap.parse_args()


def max_over_ranks(v: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time: a step of the job ends when every replica has
    finished (all_reduce MAX over the default process group)."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    if PEAKS_FILE.exists():
        d = json.loads(PEAKS_FILE.read_text())
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM, "fallback"


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def make_inputs(dims, seed, eps):
    from openstaple_gb300 import fields as F
    u = F.random_su3_links(dims, seed, eps=eps)
    ph = F.staggered_phases(dims)
    b = F.gaussian_vec3(dims, seed + 1)
    return u, ph, b


def thermalized_links(lat, dims, seed, args):
    """A thermalised configuration (outside every timed region): cold start,
    args.therm pure-gauge tree-level Symanzik HMC trajectories at args.beta
    with the reference's integrator (18 steps x 4 gauge substeps, length 1),
    FP32 molecular dynamics, the first args.therm_nometro without the
    Metropolis test; then args.stout stout steps of rho = 0.15.  Returns the
    smeared links (host su3_soa[8]) and a summary."""
    from openstaple_gb300 import api, fields as F
    from openstaple_gb300.native import act_params
    n0 = min(args.therm_nometro, args.therm)
    u, info = (None, None) if args.no_link_cache else cached_links(lat, dims, seed, args, n0)
    if u is None:
        u = F.cold_links(dims)
        lat.present(u)
        t0 = time.perf_counter()
        a = api.pure_gauge_hmc(u, args.beta, n0, 18, 4, 1.0, seed=seed, first_traj=0, precision="fp32",
                               metropolis=False)
        b = api.pure_gauge_hmc(u, args.beta, args.therm - n0, 18, 4, 1.0, seed=seed, first_traj=n0,
                               precision="fp32", metropolis=True)
        lat.sync()
        t_hmc = time.perf_counter() - t0
        plaq = np.concatenate([a["plaquette"], b["plaquette"]])
        ds = b["delta_s"]
        info = {"beta": args.beta, "trajectories": args.therm, "without_metropolis": n0,
                "accepted_with_metropolis": int(b["accepted"]), "seconds": round(t_hmc, 2),
                "plaquette_last": float(plaq[-1]) if len(plaq) else None,
                "plaquette_mean_last_50": float(plaq[-50:].mean()) if len(plaq) else None,
                "abs_delta_s_mean": float(np.abs(ds).mean()) if len(ds) else None,
                "integrator": "2MN, 18 steps x 4 gauge substeps, length 1, FP32 molecular dynamics, FP64 Metropolis",
                "seed": seed}
        lat.update_host(u)
        if not args.no_link_cache:
            store_links(u, dims, seed, args, n0, info)
    info = dict(info, stout={"steps": args.stout, "rho": 0.15})
    if args.stout > 0:
        api.set_stout_rho(0.15)
        act_params().stout_steps = args.stout
        levels = api.su3_field(lat.sizeh, 8 * args.stout)
        lat.present(levels, copy=False)
        api.stout_wrapper(u, levels, 0)
        lat.update_host(levels)
        out = levels[8 * (args.stout - 1):].copy()
        lat.release(levels)
    else:
        lat.update_host(u)
        out = u.copy()
    lat.release(u)
    return np.ascontiguousarray(out), info


def _cache_path(dims, seed, args, n0):
    root = Path(os.environ.get("OSTAPLE_LINK_CACHE", Path(tempfile.gettempdir()) / "ostaple_links"))
    tag = "tlsm_%s_b%g_t%d_n%d_s%d" % ("x".join(map(str, dims)), args.beta, args.therm, n0, seed)
    return root / (tag + ".ildg"), root / (tag + ".json")


def cached_links(lat, dims, seed, args, n0):
    """The thermalised configuration of an earlier run on this machine (the
    library's ILDG reader on a file its writer made), accepted only when its
    plaquette equals the one recorded when it was generated; else None."""
    import ctypes as C
    from openstaple_gb300 import api
    from openstaple_gb300.native import lib
    conf, meta = _cache_path(dims, seed, args, n0)
    if not (conf.exists() and meta.exists()):
        return None, None
    try:
        info = json.loads(meta.read_text())
        u = api.su3_field(lat.sizeh)
        traj = C.c_int(0)
        if lib().read_su3_soa_ildg_binary(u.ctypes.data, str(conf).encode(), C.byref(traj)) != 0:
            lib().ostaple_clear_error()
            return None, None
        lat.present(u)
        plaq = api.calc_plaquette_soloopenacc(u) / (18 * 2 * lat.sizeh)
        if abs(plaq - info["plaquette_last"]) > 1e-12:
            lat.release(u)
            return None, None
    except (OSError, ValueError, KeyError, TypeError, RuntimeError):
        return None, None
    info["read_from"] = "ILDG file written by the library after generation on this machine (plaquette checked)"
    return u, info


def store_links(u, dims, seed, args, n0, info):
    from openstaple_gb300.native import lib
    conf, meta = _cache_path(dims, seed, args, n0)
    try:
        conf.parent.mkdir(parents=True, exist_ok=True)
        if lib().print_su3_soa_ildg_binary(u.ctypes.data, str(conf).encode(), args.therm) == 0:
            meta.write_text(json.dumps(info))
        else:
            lib().ostaple_clear_error()
    except OSError:
        pass


def cpu_cg_rate(dims, u, ph, b, mass, res, fp64_iters, budget_s=20.0):
    """Times the oracle port of the reference's FP64 CG (all host threads) on a
    bounded number of iterations and extrapolates to the full solve with the
    iteration count of the identical FP64 algorithm."""
    from oracle import Oracle
    threads = os.cpu_count() or 1
    o = Oracle(dims, threads=threads)
    t0 = time.perf_counter()
    o.cg(u, ph, mass, b, res, max_cg=2, restart=2)
    per_iter = (time.perf_counter() - t0) / 2.0
    n = int(max(3, min(fp64_iters, budget_s / max(per_iter, 1e-6))))
    t0 = time.perf_counter()
    o.cg(u, ph, mass, b, res, max_cg=n, restart=n)
    per_iter = (time.perf_counter() - t0) / n
    solve_s = per_iter * fp64_iters
    return dict(value=1.0 / solve_s, unit="solves/s", cores=threads, kind="port",
                sample=f"{n} FP64 CG iterations of the oracle port on {'x'.join(map(str, dims))} "
                       f"({per_iter * 1e3:.1f} ms/iteration) x {fp64_iters} iterations per solve")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    dims = tuple(int(x) for x in args.dims.split(","))
    from oracle import Oracle
    threads = os.cpu_count() or 1
    u, ph, b = make_inputs(dims, args.seed, args.eps)
    therm = None
    if args.links_source == "thermalized":
        # the same input configuration as the GPU arm, made by the library's
        # link generator on the GPU (input data, outside the timed region);
        # without a GPU the seeded synthetic links stand in, and the line says so
        import torch
        if torch.cuda.is_available():
            from openstaple_gb300 import api
            torch.cuda.set_device(0)
            lat = api.Lattice(dims)
            u, therm = thermalized_links(lat, dims, args.seed, args)
            lat.close()
        else:
            args.links_source = "synthetic (no GPU here to generate the thermalised configuration)"
    o = Oracle(dims, threads=threads)
    times, iters = [], None
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        st, n, x = o.cg(u, ph, args.mass, b, args.res)
        dt = time.perf_counter() - t0
        iters = n
        if k >= args.warmup:
            times.append(dt)
        if k == 0 and dt * (args.warmup + args.steps) > 300:
            # bounded samples: keep the run within minutes
            args.steps, args.warmup = 1, 0
            times = [dt]
            break
    ms = 1e3 * float(np.mean(times))
    val = 1e3 / ms
    line = {"impl": "reference", "metric": "MdagM solves/s to FP64 true residual 1e-10", "value": val,
            "unit": "solves/s", "n_gpus": args.gpus, "steps": len(times), "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"MdagM CG solve {'x'.join(map(str, dims))} m={args.mass} res={args.res}",
                       "solver": "FP64 CG (inverter_full.c:19-132), oracle port, all host threads",
                       "cg_iterations": iters, "links": args.links_source, "thermalization": therm},
            "cpu_baseline": {"value": val, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": f"{len(times)} full FP64 CG solves"},
            "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    import ctypes as C
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    from openstaple_gb300 import api
    from openstaple_gb300.native import bench_lib, lib
    L = lib()
    LB = bench_lib()
    dims = tuple(int(x) for x in args.dims.split(","))
    u, ph, b = make_inputs(dims, args.seed + 17 * rank, args.eps)
    lat = api.Lattice(dims)
    therm = None
    if args.links_source == "thermalized":
        u, therm = thermalized_links(lat, dims, args.seed + 17 * rank, args)
    api.set_sloppy_links(args.links)
    bytes_deo, bytes_doe = (BYTES_Q16_DEO, BYTES_Q16_SIGN) if args.links == "q16" else (BYTES_F32_DEO, BYTES_F32_SIGN)
    stream = torch.cuda.Stream()
    L.ostaple_set_stream(C.c_void_p(stream.cuda_stream))
    x = lat.vec3()
    for a in (u, ph, b, x):
        lat.present(a)
    nrhs = max(1, args.rhs)
    if nrhs > 1:     # several right-hand sides: seeded sources, one batched solve per step
        from openstaple_gb300 import fields as F
        bs = np.stack([b] + [F.gaussian_vec3(dims, args.seed + 17 * rank + 100 + k) for k in range(nrhs - 1)])
        xs = lat.vec3(nrhs)
        lat.present(bs)
        lat.present(xs)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # plain FP64 CG (the reference algorithm on the GPU), timed once after a warm-up
    work = [lat.vec3() for _ in range(4)]
    for a in work:
        lat.present(a, copy=False)
    fp = api.make_ferm_param(args.mass, ph)
    fp64 = {"ms": None, "iters": 0, "status": -1}
    for k in range(0 if args.skip_fp64 else 2):
        L.set_vec3_soa_to_zero(x.ctypes.data)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        st, n = api.ker_invert_openacc(u, fp, x, b, args.res, *work, 100000, 0.0)
        e1.record(stream)
        torch.cuda.synchronize()
        fp64 = dict(ms=e0.elapsed_time(e1), iters=n, status=st)
    # the FP64 solution the other solvers' results are compared with
    x64 = lat.update_host(x).copy() if fp64["iters"] > 0 else None
    for a in work:
        lat.release(a)

    learned = None
    if args.solver == "learned":
        # training pairs (b_i, x_i) from the batched solver, then GPU training
        from openstaple_gb300 import fields as F
        npairs = max(1, args.pairs)
        pair_res = args.pair_res or args.res
        # sources drawn on the device (the host generator's numbers) and
        # solutions starting from zero: the host arrays are never touched
        tb = np.empty((npairs, 3, lat.sizeh), np.complex128)
        tx = np.empty((npairs, 3, lat.sizeh), np.complex128)
        lat.present(tb, copy=False)
        lat.present(tx, copy=False)
        for k in range(npairs):
            api.check(L.ostaple_gaussian_vec3(tb[k].ctypes.data, args.seed + 17 * rank + 500 + k, 7),
                      "ostaple_gaussian_vec3")
        t0 = time.perf_counter()
        for k0 in range(0, npairs, 8):
            k1 = min(npairs, k0 + 8)
            rp = api.invert_mixed_batch(u, ph, args.mass, tx[k0:k1], tb[k0:k1], None, pair_res, 100000, args.delta)
            assert rp["status"] == 1, "training pair solve failed"
        t1 = time.perf_counter()
        api.net_init(11, 0.05)
        hist = api.net_train(u, ph, args.mass, tb, tx, args.train_epochs, 3e-3)
        t2 = time.perf_counter()
        learned = {"pairs": npairs, "pair_residual": pair_res, "pair_generation_s": t1 - t0,
                   "epochs": args.train_epochs, "training_s": t2 - t1,
                   "loss_first": float(hist[0]), "loss_last": float(hist[-1])}
        lat.release(tb)
        lat.release(tx)
        del tb, tx
        # the mixed-precision CG alone on the same system, for comparison
        tm = []
        for _ in range(2):
            L.set_vec3_soa_to_zero(x.ctypes.data)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            rm = api.invert_mixed(u, ph, args.mass, 0.0, x, b, args.res, 100000, args.every, args.delta)
            e1.record(stream)
            torch.cuda.synchronize()
            tm.append(e0.elapsed_time(e1))
        learned["mixed_cg"] = {"ms": min(tm), "iterations": int(rm["iters"]), "status": int(rm["status"])}

    def solve():
        if args.solver == "learned":
            L.set_vec3_soa_to_zero(x.ctypes.data)
            r = api.invert_learned(u, ph, args.mass, 0.0, x, b, args.res, 100000)
            learned["used_fallback"] = r["used_fallback"]
            return dict(status=r["status"], iters=r["iters"], true_res=r["true_res"], n_reliable=-1)
        if nrhs > 1:
            for k in range(nrhs):
                L.set_vec3_soa_to_zero(xs[k].ctypes.data)
            r = api.invert_mixed_batch(u, ph, args.mass, xs, bs, None, args.res, 100000, args.delta)
            return dict(status=r["status"], iters=int(r["iters"].max()), true_res=float(r["true_res"].max()),
                        n_reliable=int(r["n_reliable"].max()))
        L.set_vec3_soa_to_zero(x.ctypes.data)
        return api.invert_mixed(u, ph, args.mass, 0.0, x, b, args.res, 100000, args.every, args.delta)

    # the same workload with 4 right-hand sides solved together (reported beside the headline)
    batched4 = None
    if nrhs == 1 and not args.skip_fp64 and args.solver == "mixed":
        from openstaple_gb300 import fields as F
        b4 = np.stack([b] + [F.gaussian_vec3(dims, args.seed + 17 * rank + 100 + k) for k in range(3)])
        x4 = lat.vec3(4)
        lat.present(b4)
        lat.present(x4)
        t4 = []
        for k in range(2):
            x4[...] = 0
            lat.update_device(x4)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            r4 = api.invert_mixed_batch(u, ph, args.mass, x4, b4, None, args.res, 100000, args.delta)
            e1.record(stream)
            torch.cuda.synchronize()
            t4.append(e0.elapsed_time(e1))
        lat.update_host(x4)
        batched4 = {"ms_per_solve": min(t4) / 4, "status": int(r4["status"]),
                    "true_residual_max": float(r4["true_res"].max()),
                    "err_vs_fp64": rel_diff(x4[0], x64) if x64 is not None else None}
        lat.release(b4)
        lat.release(x4)

    # the batched multi-shift workload: 4 sources x the 19 shifts of the
    # order-19 x^(-1/4) approximation (rescaled to [lambda_min, 64 * 1.05]),
    # every system to an FP64 true residual of 1e-10, against the reference
    # algorithm (multishift_invert, FP64) on the GPU, one source at a time
    multishift = None
    if nrhs == 1 and not args.skip_fp64 and args.solver == "mixed" and not args.no_multishift:
        try:
            multishift = run_multishift(api, L, lat, u, ph, b, dims, rank, stream, args)
        except Exception as exc:   # reported, never fatal to the headline line
            multishift = {"error": str(exc)[:200]}

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        for _ in range(args.warmup):
            info = solve()
        barrier()
        launches0 = L.ostaple_kernel_launches()
        e0.record(stream)
        infos = [solve() for _ in range(args.steps)]
        e1.record(stream)
        barrier()
    launches = L.ostaple_kernel_launches() - launches0
    err_vs_fp64 = None
    if x64 is not None:
        lat.update_host(xs if nrhs > 1 else x)
        err_vs_fp64 = rel_diff(xs[0] if nrhs > 1 else x, x64)
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world)
    value = world * nrhs * 1e3 / ms
    ok = all(i["status"] == 1 and i["true_res"] <= args.res for i in infos)

    # roofline of the dominant kernel of the solve (the FP32 D_eo with the
    # M^+M epilogue and <p, Ap>), and of the D_oe beside it, each timed alone
    hbm, peak_kind = peaks()
    kms = C.c_double(0)
    LB.ostaple_time_kernel(2, u.ctypes.data, ph.ctypes.data, 50, C.byref(kms))
    achieved = bytes_deo * lat.sizeh / (kms.value * 1e-3) / 1e9
    kdoe = C.c_double(0)
    LB.ostaple_time_kernel(1, u.ctypes.data, ph.ctypes.data, 50, C.byref(kdoe))
    achieved_doe = bytes_doe * lat.sizeh / (kdoe.value * 1e-3) / 1e9
    traffic, traffic_doe = None, None
    if PROFILE_TRAFFIC.exists():
        tr = json.loads(PROFILE_TRAFFIC.read_text())
        tag = 'x'.join(map(str, dims))
        fam = "q16" if args.links == "q16" else "f32"
        traffic = tr.get(f"dslash_{fam}_deo_dot_{tag}", {}).get("bytes_per_launch")
        traffic_doe = tr.get(f"dslash_{fam}_doe_{tag}", {}).get("bytes_per_launch")
    k64 = C.c_double(0)
    LB.ostaple_time_kernel(0, u.ctypes.data, ph.ctypes.data, 10, C.byref(k64))
    fp64_peak = C.c_double(0)
    LB.ostaple_probe_fma_tflops(1, C.byref(fp64_peak))
    dslash64_flops = 2 * (8 * 60 + 6) * lat.sizeh  # executed FP64 FMAs (x2) per application

    # end to end through the C entry points, from host buffers allocated
    # page-locked (copies of the inputs made before the timed region)
    e2e = None
    if not args.no_e2e:
        def pinned_copy(a):
            t = torch.empty(a.shape, dtype={np.complex128: torch.complex128, np.float64: torch.float64}[a.dtype.type],
                            pin_memory=True)
            n = t.numpy()
            n[...] = a
            return n
        xe0, be0 = (xs, bs) if nrhs > 1 else (x, b)
        ue, phe, be, xe = (pinned_copy(a) for a in (u, ph, be0, xe0))
        for a in (ue, phe, be, xe):
            lat.present(a, copy=False)
        # what the solve reads: rows 0-1 of every link (the third row is
        # rebuilt in the kernels, as in the reference), phases, source, guess
        inputs = [ue[d, 0:2] for d in range(ue.shape[0])] + [phe, be, xe]
        h2d = sum(a.nbytes for a in inputs)
        d2h = xe.nbytes
        times, phases, copies, reads = [], [], [], []
        e2e_steps = max(args.steps, 9)   # enough steps to average over both copy regimes
        for k in range(args.warmup + e2e_steps):
            xe[...] = 0
            barrier()
            t0 = time.perf_counter()
            for a in inputs:
                lat.update_device(a)
            tc = time.perf_counter()
            c0 = torch.cuda.Event(enable_timing=True)
            c0.record(stream)
            if args.solver == "learned":
                api.invert_learned(ue, phe, args.mass, 0.0, xe, be, args.res, 100000)
            elif nrhs > 1:
                api.invert_mixed_batch(ue, phe, args.mass, xe, be, None, args.res, 100000, args.delta)
            else:
                api.invert_mixed(ue, phe, args.mass, 0.0, xe, be, args.res, 100000, args.every, args.delta)
            c1 = torch.cuda.Event(enable_timing=True)
            c1.record(stream)
            tr = time.perf_counter()
            lat.update_host(xe)
            dt = time.perf_counter() - t0
            if k >= args.warmup:
                times.append(dt)
                copies.append(round(1e3 * (tc - t0), 3))
                reads.append(round(1e3 * (t0 + dt - tr), 3))
                # device time of the solve call alone (from after the copies
                # to before the read-back), to tell host stalls from GPU work
                phases.append(round(c0.elapsed_time(c1), 3))
        for a in (ue, phe, be, xe):
            lat.release(a)
        # the mean of the timed steps, i.e. the throughput of the whole run:
        # after sustained GPU load the host->device copy rate drops, so the
        # steps alternate between fast and slow copies and a median would
        # pick one regime or the other; every step is listed
        e2e_ms = max_over_ranks(1e3 * float(np.mean(times)), world)
        e2e = {"value": world * nrhs * 1e3 / e2e_ms, "unit": "solves/s", "ms_per_step": e2e_ms,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "step_ms": [round(1e3 * t, 3) for t in times], "solve_device_ms": phases,
               "h2d_host_ms": copies, "d2h_host_ms": reads,
               "statistic": "mean of the timed steps",
               "host_buffers": "page-locked (torch pin_memory)"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline and fp64["iters"] > 0:
        cpu = cpu_cg_rate(dims, u, ph, b, args.mass, args.res, fp64["iters"])

    if rank == 0:
        line = {
            "metric": "MdagM solves/s to FP64 true residual 1e-10", "value": value, "unit": "solves/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": ("synthetic: thermalised tree-level Symanzik configuration at beta=%g (library pure-gauge HMC "
                     "from a cold start, %d trajectories) + %d stout steps rho=0.15, Gaussian source"
                     % (args.beta, args.therm, args.stout) if args.links_source == "thermalized" else
                     "synthetic (seeded exp(i*0.3*H) links, Gaussian source)"),
            "config": {"workload": f"MdagM solve {'x'.join(map(str, dims))} m={args.mass} to FP64 true residual "
                                   f"{args.res}",
                       "solver": ("flexible CG preconditioned by the learned gauge-covariant network (tcgen05 BF16), "
                                  "plain CG fallback" if args.solver == "learned" else
                                  "mixed-precision CG (FP32 iteration, double-float reliable updates, FP64 final "
                                  "residual, CUDA-graph chunks)" if nrhs == 1 else
                                  f"batched mixed-precision CG, {nrhs} right-hand sides sharing each link load"),
                       "sloppy_links": args.links,
                       "learned": learned,
                       "rhs_per_step": nrhs,
                       "batched_4rhs": batched4,
                       "multishift_4x19": multishift,
                       "links": args.links_source,
                       "thermalization": therm,
                       "reliable_every": args.every,
                       "iterations": infos[-1]["iters"], "reliable_updates": infos[-1]["n_reliable"],
                       "true_residual": infos[-1]["true_res"], "all_converged": ok,
                       "err_vs_fp64": err_vs_fp64,
                       "err_vs_fp64_note": ("|x - x_fp64| / |x_fp64| of the last timed solve (of the first source "
                                            "when several are solved) against the plain FP64 CG solution of the "
                                            "same system; both have FP64 true residual <= %g, so their difference "
                                            "is bounded by the residual times the condition number, not by the "
                                            "FP32 arithmetic" % args.res),
                       "plain_fp64_cg": {"ms": fp64["ms"], "iterations": fp64["iters"], "status": fp64["status"]},
                       "speedup_vs_plain_fp64_cg": fp64["ms"] * nrhs / ms if fp64["ms"] else None,
                       "l2": ("inputs larger than L2: the FP32 iteration streams %.0f MB of 16-bit links, %.0f MB "
                              "of FP32 vectors and reads the FP64 links (%.0f MB) at reliable updates; L2 is "
                              "126 MB" % (8 * 24 * lat.sizeh / 1e6, 5 * 24 * lat.sizeh / 1e6,
                                          8 * 9 * 16 * lat.sizeh / 1e6)),
                       "parallelism": f"replicas x{world}"},
            "roofline": {"kernel": "k_mx_deo_dot (FP32 D_eo + M^+M epilogue + <p,Ap>, "
                                   + ("16-bit fixed-point links" if args.links == "q16" else "FP32 two-row links")
                                   + " + sign bytes)",
                         "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "traffic": traffic, "bytes_per_site": bytes_deo, "ms_per_launch": kms.value,
                         "doe": {"kernel": "k_mx_doe (FP32 D_oe)", "achieved": achieved_doe,
                                 "frac": achieved_doe / hbm, "traffic": traffic_doe, "bytes_per_site": bytes_doe,
                                 "ms_per_launch": kdoe.value}},
            "fp64_dslash": {"ms_per_launch": k64.value,
                            "hbm_gbs": BYTES_F64_ANGLE * lat.sizeh / (k64.value * 1e-3) / 1e9,
                            "fp64_tflops_executed": dslash64_flops / (k64.value * 1e-3) / 1e12,
                            "fp64_fma_peak_tflops_measured": fp64_peak.value},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "autotune": api.autotune_report().splitlines(),
        }
        print(json.dumps(line))
    lat.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
