"""Benchmark of the GB300 FLAC step: element-steps/s on the 1000x300-quad
two-phase extension model (config 2 of the workload list).

A "step" is one call of the reference's `flac` (fl_therm, change_phase every
ifreq_rmasses steps, fl_rheol, fl_node, fl_move, rmasses / dt_mass every
ifreq_* steps) over the whole mesh.  `value` is the FP64 path (device-resident
state, graph-replayed steps, CUDA events on the library's stream, L2 flushed
between timed steps); the mixed-precision path is reported beside it.
`e2e` drives the same steps through the per-subroutine C-ABI calls a
Fortran drop-in makes (clock scalars in, cord and vel copied back to pinned
host memory every step as the reference's OpenACC build does at
fl_move.f90:34).

--impl reference times the oracle (the serial/OpenMP FP64 restatement of the
reference's loops; the Fortran reference cannot be built on these machines)
on the host cores.

Multi-GPU: the path does not shard (one mesh per GPU); N>1 runs N
independent replicas, one per rank, and `value` sums their throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "element-steps/s on 1 GB300: FP64 vs mixed vs batched; surrogate sweep speedup @err"
WORKLOAD = ("extension_1000x300: two-phase extension, 1000x300 quads (300,000 elements, 301,301 nodes), "
            "1000 km x 300 km, 25 markers per element")
MARKERS_PER_SIDE = 5  # 5 x 5 = 25 markers per element


def bench_config(ws: int) -> dict:
    """The `config` object of both arms' JSON lines (the same workload)."""
    return {"workload": WORKLOAD, "mode": "fp64", "elements": 1000 * 300, "nodes": 1001 * 301,
            "markers_per_element": MARKERS_PER_SIDE ** 2, "parallelism": f"replicas x{ws}",
            "l2": "inputs larger than L2 between timed steps (512 MiB buffer written; host arm: n/a)"}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _max_over_ranks(x: float, device: str) -> float:
    """The largest value of x over the ranks of the process group (x itself
    without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _replica_throughput(units_per_rank: float, t_rank: float, device: str):
    """Whole-job throughput of N independent replicas: all ranks' units over
    the slowest rank's time.  Returns (value, slowest time)."""
    import torch.distributed as dist

    ws = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    t = _max_over_ranks(t_rank, device)
    return ws * units_per_rank / t, t


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def _ncu_pipe(kernel: str):
    """(pipe, fraction of its peak) of `kernel` from the committed ncu summary,
    if any: the compute bound of a kernel that HBM does not bound."""
    path = os.path.join(ROOT, "profiles", "pipes.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and parts[0] == kernel:
            try:
                return {"pipe": parts[1], "frac_of_peak": float(parts[2]), "source": "ncu (profiles/)"}
            except ValueError:
                return None
    return None


def _make_model(inp: str, mode: str):
    import torch

    from geoflac_gb300 import new_state
    from geoflac_gb300.flac import Flac

    p, c, s = new_state(inp, markers_per_side=MARKERS_PER_SIDE)
    bufs = []

    def pinned(nbytes):
        t = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        bufs.append(t)
        return t.numpy()

    # the arrays the drop-in path copies every step live in pinned memory
    s.rehome(["cord", "vel"], pinned)
    g = Flac(p, c, s, mode)
    g._pinned = bufs
    return g


def _time_device(g, steps: int, warmup: int, flush):
    """Per-step device time with CUDA events on the library's stream, L2
    flushed (a 512 MiB write) before each timed step."""
    import torch

    stream = torch.cuda.ExternalStream(g.stream)
    g.step(warmup)
    torch.cuda.synchronize()
    total = 0.0
    launches0 = g.launches
    t0 = time.perf_counter()
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        g.step(1)
        ev1.record(stream)
        ev1.synchronize()
        total += ev0.elapsed_time(ev1) / 1e3
    wall = time.perf_counter() - t0
    return total, g.launches - launches0, wall


def _time_kernel(g, routine: str, reps: int, flush):
    """Average duration of one routine's kernels (CUDA events on the stream)."""
    import torch

    stream = torch.cuda.ExternalStream(g.stream)
    g.set_sync(False)
    times = []
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        getattr(g, routine)()
        ev1.record(stream)
        ev1.synchronize()
        times.append(ev0.elapsed_time(ev1) / 1e3)
    g.set_sync(True)
    g.status()
    return sum(times) / len(times)


def _time_e2e(g, steps: int):
    """Drop-in path: per-subroutine C-ABI calls with the reference's host
    synchronisation (clock scalars in/out, cord+vel back every step)."""
    import ctypes as C

    import torch

    from geoflac_gb300 import capi

    p = g.params
    N = p.nx * p.nz
    lib = g.lib
    k = capi.GfClock()
    capi.check(lib.gf_get_clock(g.ctx, C.byref(k)), "gf_get_clock")
    g.set_sync(False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        capi.check(lib.gf_set_clock(g.ctx, C.byref(k)), "gf_set_clock")
        g.fl_therm()
        if k.nloop % p.ifreq_rmasses == 0:
            g.change_phase()
        g.fl_rheol()
        g.fl_node()
        g.fl_move()
        if k.nloop % p.ifreq_rmasses == 0:
            g.rmasses()
        if k.nloop % p.ifreq_imasses == 0:
            g.dt_mass()
        # par.f90:84-87 on the host: read dt back, advance nloop and time
        capi.check(lib.gf_get_clock(g.ctx, C.byref(k)), "gf_get_clock")
        k.nloop += 1
        k.time += k.dt
        # the reference copies cord and vel to the host every step; the
        # host arrays are pinned
        capi.check(lib.gf_download(g.ctx, capi.F_CORD | capi.F_VEL), "gf_download")
    capi.check(lib.gf_set_clock(g.ctx, C.byref(k)), "gf_set_clock")
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    g.set_sync(True)
    g.status()
    h2d = C.sizeof(capi.GfClock)
    d2h = 4 * N * 8 + C.sizeof(capi.GfClock)
    return wall, h2d, d2h


def run_ours(args):
    import torch

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from geoflac_gb300 import bytes_model, inpgen

    d = tempfile.mkdtemp(prefix="gfbench")
    inp = inpgen.extension_1000x300().write(os.path.join(d, "extension_1000x300.inp"))
    if args.profile in ("fno", "batch", "magma"):
        profile_extra(args, d)
        return
    if args.profile:
        # profiling run: only `warmup + steps` graph-replayed steps of one mode
        g = _make_model(inp, args.profile)
        g.step(args.warmup + args.steps)
        g.status()
        print(json.dumps({"profile": args.profile, "steps": args.warmup + args.steps, "launches": g.launches}))
        g.close()
        return
    if args.only == "surrogate":  # development: the surrogate leg alone
        args.batch_cfg = dict(threads=256, items_per_thread=2, ctas_per_sm=2, graph_steps=10)
        print(json.dumps({"metric": METRIC, "partial": "surrogate leg only",
                          "surrogate": bench_surrogate(args, d)}))
        return
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    E = 1000 * 300
    res = {}
    for mode in ("fp64", "mixed"):
        g = _make_model(inp, mode)
        with ClockSampler(local) as cs:
            if ws > 1:
                dist.barrier()
            torch.cuda.synchronize()
            dev_t, launches, wall = _time_device(g, args.steps, args.warmup, flush)
            torch.cuda.synchronize()
        dev_t = _max_over_ranks(dev_t, "cuda")
        res[mode] = dict(g=g, t=dev_t, launches=launches, clocks=cs.summary(), wall=wall)
    fp = res["fp64"]
    # both modes advanced the same number of steps from the same state:
    # per-field error of the mixed path, max|a-b| / max|b|
    mixed_err = {}
    fp["g"].download()
    res["mixed"]["g"].download()
    for f in ("vel", "cord", "temp", "stress0", "aps"):
        a, b = res["mixed"]["g"].state[f], fp["g"].state[f]
        mixed_err[f] = float(abs(a - b).max() / max(abs(b).max(), 1e-300))
    # the model's own sensitivity: the FP64 run from an initial stress
    # perturbed by a relative 1e-7 (FP32 rounding), same steps
    import numpy as np

    from geoflac_gb300 import capi as _capi

    gp = _make_model(inp, "fp64")
    st = gp.download(_capi.F_STRESS)["stress0"]
    st[...] = st * (1.0 + 1e-7 * np.random.default_rng(7).standard_normal(st.shape))
    gp.upload(_capi.F_STRESS)
    gp.step(args.warmup + args.steps)
    gp.download()
    perturbed_err = {}
    for f in ("vel", "cord", "temp", "stress0", "aps"):
        a, b = gp.state[f], fp["g"].state[f]
        perturbed_err[f] = float(abs(a - b).max() / max(abs(b).max(), 1e-300))
    gp.close()
    value = ws * E * args.steps / fp["t"]
    mixed_value = ws * E * args.steps / res["mixed"]["t"]
    # dominant kernel: fl_rheol (k_rheol), timed alone
    g = fp["g"]
    t_rheol = _time_kernel(g, "fl_rheol", 10, flush)
    peak, peak_kind = _peaks()
    alg = bytes_model.rheol_bytes_per_element(g.params.nphase, "fp64") * E
    achieved = alg / t_rheol / 1e9
    traffic = _ncu_traffic("k_rheol_fp64")
    # the mixed path's dominant kernel (k_rheol<float>), timed alone
    gm = res["mixed"]["g"]
    t_rheol_m = _time_kernel(gm, "fl_rheol", 10, flush)
    alg_m = bytes_model.rheol_bytes_per_element(gm.params.nphase, "mixed") * E
    mixed_roofline = {"bound": "hbm", "kernel": "k_rheol (fl_rheol, mixed)", "achieved": alg_m / t_rheol_m / 1e9,
                      "peak": peak, "unit": "GB/s", "frac": alg_m / t_rheol_m / 1e9 / peak, "peak_kind": peak_kind,
                      "traffic": _ncu_traffic("k_rheol_mixed"), "avg_launch_s": t_rheol_m,
                      "algorithmic_bytes_per_launch": alg_m}
    # e2e through the per-subroutine C-ABI (drop-in path)
    e2e_steps = max(5, min(args.steps, 20))
    e2e_wall, h2d, d2h = _time_e2e(g, e2e_steps)
    e2e_value = ws * E * e2e_steps / e2e_wall
    e2e = {"value": e2e_value, "unit": "element-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "steps": e2e_steps,
           "path": "per-subroutine C-ABI calls, clock scalars in/out, cord+vel to host every step"}
    roofline = {"bound": "hbm", "kernel": "k_rheol (fl_rheol, FP64)", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                "avg_launch_s": t_rheol, "algorithmic_bytes_per_launch": alg, "compute": _ncu_pipe("k_rheol_fp64")}
    for r in res.values():
        r["g"].close()
    err10 = mixed_error_steps(inp, 10)
    detail = {"mixed_rel_err_vs_fp64": mixed_err, "mixed_err_after_steps": args.steps + args.warmup,
              "mixed_rel_err_vs_fp64_10_steps": err10, "fp64_perturbed_1e-7_rel_err": perturbed_err,
              "mixed_roofline": mixed_roofline, "e2e": e2e, "roofline": roofline,
              "therm_sweeps_fp64": fp["g"].clock.therm_sweeps, "clocks_mixed": res["mixed"]["clocks"]}
    out = {
        "metric": METRIC, "value": value, "unit": "element-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * fp["t"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded .inp model)",
        "config": bench_config(ws),
        "e2e": {k: e2e[k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step")},
        "roofline": {k: _r(roofline[k]) for k in ("bound", "achieved", "peak", "unit", "frac", "traffic", "compute")},
        "gpu_launches": fp["launches"],
        "clocks": {k: fp["clocks"].get(k) for k in ("sm_mhz", "sm_max_mhz", "reasons")},
        "mixed": {"value": _r(mixed_value), "ms_per_step": _r(1e3 * res["mixed"]["t"] / args.steps),
                  "speedup_vs_fp64": _r(mixed_value / value),
                  "vel_rel_err_vs_fp64": {"10_steps": _r(err10["vel"]), f"{args.steps + args.warmup}_steps":
                                          _r(mixed_err["vel"])},
                  "fp64_own_vel_change_1e-7": _r(perturbed_err["vel"]),
                  "roofline_frac": _r(mixed_roofline["frac"])},
    }
    if args.members > 0:
        bt = bench_batch(args, d, local)
        detail["batched"] = dict(bt)
        out["batched"] = {"value": _r(bt["value"]), "ms_per_step": _r(bt["ms_per_step"]), "members": bt["members"],
                          "elements": bt["elements"], "roofline_frac": _r(bt["roofline"]["frac"]),
                          "config": bt["config"]}
        if args.sur_epochs > 0:
            args.batch_cfg = {k: v for k, v in bt["config"].items()}
            sg = bench_surrogate(args, d)
            detail["surrogate"] = sg
            out["surrogate"] = {"speedup_vs_plain": _r(sg["speedup_vs_plain"]),
                                "screen_s": _r(sg["screen_seconds"]), "plain_s": _r(sg["plain_seconds"]),
                                "rerun_members": sg["rerun_members"],
                                "rel_err": {k: {q: _r(v) for q, v in sg["rel_err"][k].items()}
                                            for k in ("topography", "plastic_strain")},
                                "members_over_2pct": sg["members_over_2pct"]}
    c1 = bench_config1(d)
    detail["config1"] = c1
    out["config1"] = {k: c1[k] for k in ("fp64", "mixed", "unit")}
    if args.c3_steps > 0:
        c3 = bench_config3(args, d)
        detail["config3"] = c3
        out["config3"] = {k: c3[k] for k in ("steps", "ms_per_step_fp64", "ms_per_step_mixed", "rel_err_vs_fp64",
                                             "fp64_own_change_1e-7", "status")}
    if rank == 0 and ws == 1 and not args.no_cpu:
        cb = cpu_baselines(inp, args)
        detail["cpu_baselines"] = cb
        out["cpu_baseline"] = dict(cb["extension_1000x300"]["all_cores"])
        out["cpu_baseline"]["value_1_thread"] = _r(cb["extension_1000x300"]["1_thread"]["value"])
        out["cpu_baseline"]["extension_60x20"] = {k: _r(v["value"]) for k, v in cb["extension_60x20"].items()}
    if rank == 0:
        # details first (an earlier line), the compact record last
        print(json.dumps({"detail": detail}))
        print(json.dumps(out))
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def _r(x, digits=4):
    """Round floats to `digits` significant digits for the compact record."""
    if isinstance(x, float):
        return float(f"{x:.{digits}g}")
    return x


def _field_errors(a, b, fields=("vel", "cord", "temp", "stress0", "aps")):
    """max |a - b| / max |b| per field"""
    return {f: float(abs(a[f] - b[f]).max() / max(abs(b[f]).max(), 1e-300)) for f in fields}


def mixed_error_steps(inp: str, steps: int):
    """Per-field error of the mixed path against the FP64 path, both advanced
    `steps` steps from the same start-up state of the bench's model."""
    a, b = _make_model(inp, "fp64"), _make_model(inp, "mixed")
    a.step(steps)
    b.step(steps)
    err = _field_errors(b.download(), a.download())
    a.close()
    b.close()
    return err


def bench_config1(workdir: str, steps: int = 2000):
    """The 60x20 extension model (1,200 elements; config 1 of the workload
    list) over its full 2000 steps, FP64 and mixed, graph-replayed steps
    timed with CUDA events: a mesh this small is bound by launch and
    synchronisation latency, not by the kernels' work."""
    import torch

    from geoflac_gb300 import inpgen, new_state
    from geoflac_gb300.flac import Flac

    inp = inpgen.extension_60x20().write(os.path.join(workdir, "extension_60x20.inp"))
    out = {"workload": "extension_60x20 (1,200 elements, 9 markers per element)", "steps": steps,
           "unit": "element-steps/s"}
    for mode in ("fp64", "mixed"):
        g = Flac(*new_state(inp), mode)
        stream = torch.cuda.ExternalStream(g.stream)
        g.step(10)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.step(steps)
        e1.record(stream)
        e1.synchronize()
        g.status()
        t = e0.elapsed_time(e1) / 1e3
        out[mode] = _r(1200 * steps / t)
        out[f"ms_per_step_{mode}"] = _r(1e3 * t / steps)
        g.close()
    return out


def bench_config3(args, workdir: str):
    """The convergent workload (600x150 quads, 1200 km x 300 km: 60-Myr
    oceanic plate with basalt and weak sediment, continental plate, left wall
    at 5 cm/yr, Winkler base, basalt -> eclogite above 600 C and 1.5 GPa)
    advanced `--c3-steps` steps in FP64 and in mixed precision from the same
    start; per-field error of the mixed run against the FP64 run, beside the
    FP64 run's own change when its initial stresses are perturbed by a
    relative 1e-7 (FP32 rounding size)."""
    import numpy as np
    import torch

    from geoflac_gb300 import inpgen, new_state
    from geoflac_gb300.flac import Flac

    inp = inpgen.convergence(600, 150).write(os.path.join(workdir, "convergence_600x150.inp"))
    steps = args.c3_steps
    fields = ("vel", "cord", "temp", "stress0", "aps")
    states, times, status = {}, {}, "ok"
    for tag, mode, perturb in (("fp64", "fp64", False), ("mixed", "mixed", False), ("fp64_pert", "fp64", True)):
        p, c, s = new_state(inp, eclogite_rule=1)
        if perturb:
            st = s["stress0"]
            st[...] = st * (1.0 + 1e-7 * np.random.default_rng(7).standard_normal(st.shape))
        g = Flac(p, c, s, mode)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            g.step(steps)
            g.status()
        except Exception as e:  # a stop code of the reference (e.g. 40: negative area)
            status = f"{tag}: {e}"
        torch.cuda.synchronize()
        times[tag] = (time.perf_counter() - t0) / steps
        st = g.download()
        states[tag] = {f: st[f].copy() for f in fields}
        states[tag]["topography"] = st["cord"][0, :, 1].copy()
        states[tag]["iphase"] = st["iphase"].copy()
        states[tag]["nloop"] = g.clock.nloop
        states[tag]["eclogite_markers"] = int(np.count_nonzero(st["mark_phase"][:g.clock.nmarkers] == 13))
        g.close()

    def errs(a, b):
        e = _field_errors(a, b, fields + ("topography",))
        e["iphase_differs"] = float(np.mean(a["iphase"] != b["iphase"]))
        return {k: _r(v) for k, v in e.items()}

    return {"workload": "convergence_600x150 (90,000 elements, eclogite at 600 C / 1.5 GPa, Winkler base)",
            "steps": steps, "status": status, "ms_per_step_fp64": _r(1e3 * times["fp64"]),
            "ms_per_step_mixed": _r(1e3 * times["mixed"]),
            "rel_err_vs_fp64": errs(states["mixed"], states["fp64"]),
            "fp64_own_change_1e-7": errs(states["fp64_pert"], states["fp64"]),
            "eclogite_markers": {k: v["eclogite_markers"] for k, v in states.items()},
            "nloop": {k: v["nloop"] for k, v in states.items()}}


def bench_batch(args, workdir: str, local: int):
    """The 256-member mixed-precision sweep (config 4 of the workload list)
    advanced by the ensemble driver: autotuned, then `args.steps` steps timed
    with CUDA events on the batch's stream (working set of several GB, far
    above L2)."""
    import torch

    from geoflac_gb300 import bytes_model
    from geoflac_gb300.batch import Batch, ensemble

    t0 = time.time()
    members = ensemble(args.members, workdir)
    setup_s = time.time() - t0
    models = [m for m, _ in members]
    b = Batch(models)
    tuned = b.tune(trial_steps=2)
    b.step(args.warmup)
    stream = torch.cuda.ExternalStream(b.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()
    with ClockSampler(local) as cs:
        e0.record(stream)
        b.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    E = b.elements
    # N replicas of the sweep (one per GPU): all ranks' element-steps over
    # the slowest rank's time
    value, t = _replica_throughput(E * args.steps, e0.elapsed_time(e1) / 1e3, "cuda")
    nodes = sum(m.params.nx * m.params.nz for m in models)
    bpe = bytes_model.step_bytes_per_element("mixed", nphase=models[0].params.nphase, n_over_e=nodes / E)
    peak, peak_kind = _peaks()
    achieved = bpe * E * args.steps / t / 1e9
    out = {"value": value, "unit": "element-steps/s", "members": len(models), "elements": E,
           "nodes": nodes, "ms_per_step": 1e3 * t / args.steps, "steps": args.steps, "dtype": "f32 element fields / f64 nodes",
           "config": {k: v for k, v in tuned.items() if k != "ms_per_step"}, "grid_ctas": b.grid,
           "gpu_launches": args.steps,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_kind": peak_kind,
                        "algorithmic_bytes_per_element_step": bpe},
           "setup_s": setup_s, "clocks": cs.summary()}
    b.close()
    for m in models:
        m.close()
    return out


def bench_surrogate(args, workdir: str):
    """Surrogate leg: snapshots of a training sweep (2048 members, 5
    snapshots each) from the ensemble driver, FNO training (the library's
    tcgen05 kernels), then screening of a fresh 256-member sweep over
    `interval` steps against the plain ensemble step of the same members
    (timed on the same GPU)."""
    import numpy as np
    import torch

    from geoflac_gb300 import surrogate as S
    from geoflac_gb300.batch import Batch, ensemble
    from geoflac_gb300.fno import FnoConfig

    cfg = FnoConfig()
    n, interval = args.members, args.sur_interval
    nt = args.sur_train_members
    t0 = time.time()
    tr = ensemble(nt, workdir)
    tb = Batch([m for m, _ in tr])
    tb.set_config(**args.batch_cfg)
    snaps = S.generate(tb, [p for _, p in tr], n_snap=args.sur_snaps, interval=interval, H=cfg.H, W=cfg.W)
    cal = S.calibrate_tolerance(tb, cfg.H, cfg.W)
    t_data = time.time() - t0
    sur = S.Surrogate(cfg, S.Normaliser.fit(snaps), seed=0)
    info = sur.train(snaps, epochs=args.sur_epochs, batch=64, lr=args.sur_lr)
    pairs = nt * (args.sur_snaps - 1)
    del snaps
    tb.close()
    for m, _ in tr:
        m.close()
    # fresh sweep, two identical copies: plain truth and screened
    d2 = os.path.join(workdir, "fresh")
    os.makedirs(d2, exist_ok=True)
    fa = ensemble(n, d2, seed=S_SEED_FRESH)
    fb = ensemble(n, d2, seed=S_SEED_FRESH)
    ba, bb = Batch([m for m, _ in fa]), Batch([m for m, _ in fb])
    for b in (ba, bb):
        b.set_config(**args.batch_cfg)
    ba.step(args.sur_start)
    bb.step(args.sur_start)
    stream = torch.cuda.ExternalStream(ba.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ba.step(interval)
    e1.record(stream)
    torch.cuda.synchronize()
    t_plain = e0.elapsed_time(e1) / 1e3
    truth = torch.empty((n, cfg.H, cfg.W, S.NCH), dtype=torch.float32, device="cuda")
    ba.sample(truth, cfg.H, cfg.W, S.CRUST_PHASE)
    torch.cuda.synchronize()
    res = S.screen(bb, sur, [p for _, p in fb], interval, cal["tol"])
    err = S.rel_errors(res["fields"], truth, res["raw_t"])
    out = {"members": n, "training_members": nt, "snapshots_per_member": args.sur_snaps,
           "interval_steps": interval, "grid": [cfg.H, cfg.W], "width": cfg.C,
           "modes": [cfg.m1, cfg.m2], "layers": cfg.layers, "training_pairs": pairs, "epochs": args.sur_epochs,
           "train_seconds": info["seconds"], "train_loss_first": info["first_loss"],
           "train_loss_final": info["final_loss"], "data_seconds": t_data,
           "plain_seconds": t_plain, "screen_seconds": res["seconds"],
           "screen_breakdown": {k[8:]: v for k, v in res.items() if k.startswith("seconds_")},
           "rerun_members": len(res["rerun"]), "rerun_detail": res["rerun_detail"],
           "rerun_elements": [int((fb[k][0].params.nx - 1) * (fb[k][0].params.nz - 1)) for k in res["rerun"]],
           "speedup_vs_plain": t_plain / res["seconds"],
           "gate": {k: v for k, v in cal.items()},
           "rel_err": {k: {"median": float(np.median(v)), "p90": float(np.quantile(v, 0.9)), "max": float(np.max(v))}
                       for k, v in err.items()},
           "members_over_2pct": {k: int(np.count_nonzero(err[k] > 0.02)) for k in ("topography", "plastic_strain")},
           # per member: the 4 sweep parameters, elements, gate residual,
           # rerun, relative L2 error of topography and plastic strain
           "per_member": [[round(float(v), 4) for v in (pp["friction"], pp["crust_km"], pp["moho_t"], pp["v_cm_yr"])] +
                          [int((fb[k][0].params.nx - 1) * (fb[k][0].params.nz - 1)),
                           float(res["residual"][k]), int(k in res["rerun"]),
                           float(err["topography"][k]), float(err["plastic_strain"][k])]
                          for k, pp in enumerate(p for _, p in fb)]}
    for b in (ba, bb):
        b.close()
    for m, _ in fa + fb:
        m.close()
    return out


S_SEED_FRESH = 20261204


def profile_extra(args, workdir: str):
    """Profiling runs of the ensemble driver and the surrogate (for ncu):
    batch = `warmup + steps` steps of a `--members` sweep; fno = `warmup +
    steps` training steps of the full-size FNO (batch 64, 128 x 384) on
    synthetic fields."""
    import numpy as np
    import torch

    if args.profile == "magma":
        return profile_magma(args, workdir)
    if args.profile == "batch":
        from geoflac_gb300.batch import Batch, ensemble

        ms = ensemble(args.members, workdir)
        b = Batch([m for m, _ in ms])
        # the autotuner's build on the 256-member sweep (256 threads, 3 CTAs
        # per SM); 2 items per thread so that a small sweep fills the grid
        b.set_config(threads=256, items_per_thread=2, ctas_per_sm=3, graph_steps=0)
        b.step(args.warmup + args.steps)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "batch", "members": args.members, "elements": b.elements,
                          "steps": args.warmup + args.steps}))
        return
    from geoflac_gb300.fno import Fno, FnoConfig

    cfg = FnoConfig()
    net = Fno(cfg, seed=0)
    rng = np.random.default_rng(0)
    nb = args.fno_batch
    x = torch.from_numpy(rng.standard_normal((nb, cfg.H, cfg.W, cfg.cin)).astype(np.float32)).cuda().to(torch.bfloat16)
    t = torch.from_numpy(rng.standard_normal((nb, cfg.H, cfg.W, cfg.cout)).astype(np.float32)).cuda()
    for _ in range(args.warmup + args.steps):
        out = net.forward(x, train=True)
        loss, dout = net.loss_grad(out, t)
        net.backward(dout)
        net.adam(lr=1e-4)
    torch.cuda.synchronize()
    print(json.dumps({"profile": "fno", "steps": args.warmup + args.steps, "loss": loss.item()}))


def _seed_melting(p, s):
    """Melting set-up of the arc model, by fractions of the mesh: a hot
    mantle column (MOR melt), subducted basalt / sediment below the Moho
    (arc melt), serpentinite under hot mantle (flux melting)."""
    import numpy as np

    nz1, nx1 = p.nz - 1, p.nx - 1
    r = lambda f: int(round(f * nz1))
    c = lambda f: int(round(f * nx1))
    T = s["temp"]
    T[r(2 / 15):r(5 / 15), c(8 / 60):c(17 / 60)] = 1500.0
    ids, nm, ph = s["mark_id_elem"], s["nmark_elem"], s["mark_phase"]
    touched = []
    for i in range(c(34 / 60), c(38 / 60)):
        for j in range(r(3 / 15), r(5 / 15)):
            ph[ids[:nm[j, i], j, i] - 1] = 3 if i % 2 else 11
            touched.append((j, i))
    T[r(3 / 15):r(6 / 15), c(34 / 60):c(39 / 60)] = 1100.0
    j0, i0 = r(6 / 15), c(45 / 60)
    ph[ids[:nm[j0, i0], j0, i0] - 1] = 9
    touched.append((j0, i0))
    T[r(3 / 15):r(7 / 15), i0:i0 + 2] = 1000.0
    for j, i in touched:  # count_phase_ratio of the changed elements
        cnt = np.bincount(ph[ids[:nm[j, i], j, i] - 1], minlength=p.nphase + 1)[1:p.nphase + 1]
        s["phase_ratio"][:, j, i] = cnt / nm[j, i]
        s["iphase"][j, i] = int(np.argmax(cnt)) + 1


def profile_magma(args, workdir: str):
    """The magma sub-model's cost: FP64 steps of the 600x150 arc model with
    melting seeded, itype_melting 1 against the same model with 0."""
    import torch

    from geoflac_gb300 import clone, inpgen, new_state
    from geoflac_gb300.flac import Flac

    m = inpgen.magma_arc(600, 150)
    # production rates of the reference's defaults: the test model's faster
    # MOR eruption lifts 2 km surface elements past their neighbours
    m.prod_magma, m.prod_magma2 = 2e-15, 1e-13
    p, c, s = new_state(m.write(os.path.join(workdir, "magma_arc.inp")))
    _seed_melting(p, s)
    p0, c0, s0 = clone(p, c, s)
    p0.itype_melting = 0
    out = {"profile": "magma", "model": "magma_arc 600x150 (convergence with 19 phases, itype_melting 1, "
                                        "prod_magma 2e-15, prod_magma2 1e-13)",
           "elements": (p.nx - 1) * (p.nz - 1), "steps": args.steps}
    for tag, (pp, cc, ss) in (("plain", (p0, c0, s0)), ("magma", (p, c, s))):
        g = Flac(pp, cc, ss, "fp64")
        g.step(args.warmup)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.step(args.steps)
        g.status()
        torch.cuda.synchronize()
        out[f"ms_per_step_{tag}"] = (time.perf_counter() - t0) * 1e3 / args.steps
        st = g.download()
        out[f"melting_elements_{tag}"] = int(((st["fmelt"] > 0) | (st["fmelt2"] > 0)).sum())
        out[f"magma_elements_{tag}"] = int(((st["fmagma"] > 0) | (st["fmagma2"] > 0)).sum())
        out[f"markers_{tag}"] = int(g.clock.nmarkers)
        g.close()
    out["overhead"] = out["ms_per_step_magma"] / out["ms_per_step_plain"]
    print(json.dumps(out))


def _oracle_rate(inp: str, steps: int, threads: int):
    """Element-steps/s of the oracle (the FP64 restatement of the reference's
    loops, OpenMP where the reference has `!$OMP do`) on `threads` host
    threads over `steps` steps after one untimed step, from its own start-up."""
    from oracle.oracle import Oracle, new_state

    p, c, s = new_state(inp, markers_per_side=MARKERS_PER_SIDE)
    o = Oracle(p, c, s, threads=threads)
    o.finish_setflac()
    o.step(1)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    return (p.nx - 1) * (p.nz - 1) * steps / dt, dt


def cpu_baselines(inp: str, args):
    """The host baseline on 1 thread and on all cores, on the bench's
    1000x300 model (bounded samples: `--cpu-steps` steps on all cores,
    a quarter of that, at least 2, on one thread) and on the 60x20 model of
    the same physics (its full 2000 steps)."""
    from geoflac_gb300 import inpgen

    n = os.cpu_count() or 1
    out = {}
    small = inpgen.extension_60x20().write(os.path.join(os.path.dirname(inp), "extension_60x20.inp"))
    for name, path, st_all, st_one in (("extension_1000x300", inp, args.cpu_steps, max(2, args.cpu_steps // 4)),
                                       ("extension_60x20", small, 2000, 2000)):
        out[name] = {}
        for tag, threads, steps in (("1_thread", 1, st_one), ("all_cores", n, st_all)):
            v, dt = _oracle_rate(path, steps, threads)
            out[name][tag] = {"value": _r(v), "unit": "element-steps/s", "cores": threads, "kind": "port",
                              "sample": f"{steps} FLAC steps of {name}, {threads} OpenMP thread(s), {dt:.1f} s"}
    return out


def run_reference(args):
    """The reference arm: the oracle (the FP64 restatement of the
    reference's loops; the Fortran reference cannot be built on these
    machines) from its own start-up state, on all host cores, with the same
    config as the GPU arm."""
    ws, rank, local = _dist()
    if rank != 0:
        return
    from geoflac_gb300 import inpgen
    from oracle.oracle import Oracle, new_state

    d = tempfile.mkdtemp(prefix="gfbench")
    inp = inpgen.extension_1000x300().write(os.path.join(d, "extension_1000x300.inp"))
    n = os.cpu_count() or 1
    p, c, s = new_state(inp, markers_per_side=MARKERS_PER_SIDE)
    o = Oracle(p, c, s, threads=n)
    o.finish_setflac()
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    E = (p.nx - 1) * (p.nz - 1)
    v = E * args.steps / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "element-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded .inp model)",
        "config": bench_config(ws),
        "cpu_baseline": {"value": v, "unit": "element-steps/s", "cores": n, "kind": "port",
                         "sample": f"{args.steps} full FLAC steps of the 1000x300 mesh, {n} OpenMP threads"},
        "e2e": {"value": v, "unit": "element-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=400, help="host baseline sample on all cores (1000x300 steps)")
    ap.add_argument("--c3-steps", type=int, default=15000, help="steps of the convergent 600x150 leg (0: skip)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--members", type=int, default=256, help="ensemble size of the batched leg (0: skip)")
    ap.add_argument("--sur-epochs", type=int, default=20, help="surrogate training epochs (0: skip the surrogate)")
    ap.add_argument("--sur-train-members", type=int, default=2048, help="members of the training sweep")
    ap.add_argument("--sur-snaps", type=int, default=5,
                    help="snapshots per training member (pairs = members x (snaps - 1))")
    ap.add_argument("--sur-interval", type=int, default=500, help="steps between snapshots and of the forecast")
    ap.add_argument("--sur-start", type=int, default=1000, help="plain steps of the fresh sweep before the forecast")
    ap.add_argument("--sur-lr", type=float, default=2e-3)
    ap.add_argument("--fno-batch", type=int, default=64, help="batch of the fno profiling run")
    ap.add_argument("--only", choices=["surrogate"], default=None, help="run one leg only (development)")
    ap.add_argument("--profile", choices=["fp64", "mixed", "batch", "fno", "magma"], default=None,
                    help="run warmup+steps steps of one mode and nothing else (for ncu)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
