#!/usr/bin/env python
"""Benchmark of the lattice evolution hot path on GB300.

Workload (one "step" = one leapfrog step of the whole lattice): Abelian-Higgs,
512^3 periodic, lambda=2, e=1, eta=1, dx=0.5, dt=0.1, PRS expansion friction
alpha=3 (a ~ tau, tau0=1), energy + Gauss diagnostics every 20 steps, seeded
uniform-phase ICs (mt19937, as mpi_evolution.cpp:287-312).  The plain FP64
path is the headline; the FP32 form is measured in the same run.

Reported (one JSON line on rank 0):
  value        site-updates/s with the state resident in HBM (CUDA events on the
               library's stream around the K timed steps);
  e2e          the same metric through the C ABI with host buffers: one
               lat_run call (upload of the initial level from pinned memory,
               a stationary start whose two levels are one array as the
               reference's IC; the K steps; the diagnostics; the download of
               the final level), all inside the timed region;
  roofline     dominant kernel (the step kernel): algorithmic bytes per
               site-update x sites / its average launch time, against the
               measured HBM copy bandwidth;
  cpu_baseline the oracle's CPU restatement (same arithmetic as the reference)
               on all host cores, on a bounded sample of the workload.

--impl reference times that CPU implementation alone for the same metric.
Multi-GPU: independent replicas (the path is not sharded), one per rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DIAG_EVERY = 20
# Workloads: "ah" (AH 512^3, the headline) and "moore" (Moore 768^3 FP32 with FP64 reductions).
MODEL = {"name": "ah"}
# Forms: "f64" is the plain FP64 path (two-pass step, fused multiply-adds, LAT_F64_FAST); "f64_strict"
# the same step in the reference's operation order (LAT_F64); "f32" FP32 fields with FP64 reductions.
FORMS = ("f64", "f64_strict", "f32")
E2E_RUNS = 3  # end-to-end runs per measurement (median reported)

# algorithmic bytes per site-update: each field value read at levels n and n-1, written at n+1
BYTES = {"ah": {"f64": 120, "f64_strict": 120, "f32": 60}, "moore": {"f64": 168, "f64_strict": 168, "f32": 84}}
KERNEL_NAME = {"f64": "ah_links_kernel + ah_update_kernel (FP64 two-pass step, fused multiply-adds)",
               "f64_strict": "ah_links_kernel + ah_update_kernel (FP64 two-pass step, reference operation order)",
               "f32": "pair_step_kernel<1> (FP32 step, two z-sites per thread in paired FP32 instructions)"}
KERNEL_NAME_MOORE = {"f64": "moore_step_kernel<double> (one-pass FP64 step)",
                     "f64_strict": "moore_step_kernel<double> (one-pass FP64 step)",
                     "f32": "pair_step_kernel<2> (FP32 step, two z-sites per thread in paired FP32 instructions, two scalars)"}


def bytes_per_site(precision: str) -> int:
    return BYTES[MODEL["name"]][precision]


def kernel_name(precision: str) -> str:
    return (KERNEL_NAME_MOORE if MODEL["name"] == "moore" else KERNEL_NAME)[precision]


def lat_precision(precision: str) -> int:
    from axions_gb300.params import F32, F64, F64_FAST
    return {"f64": F64_FAST, "f64_strict": F64, "f32": F32}[precision]


def workload_params(n: int, precision: str):
    from axions_gb300.params import ENERGY_EVOLUTION, MODEL_MOORE, make_params
    prec = lat_precision(precision)
    if MODEL["name"] == "moore":
        return moore_params(n, precision)
    return make_params(0, n=n, d=0.5, dt=0.1, lam=2.0, eta=1.0, g=1.0, damped_nt=0, dampFac=0.0, alpha=3.0,
                       scaling=1.0, tau0=1.0, energy_form=ENERGY_EVOLUTION, precision=prec)


def moore_params(n: int, precision: str):
    """Config 3: two scalars with charges 1 and 2, equal vevs, lambda1 =
    lambda2 = 2, e = 1, dx = 0.5, dt = 0.1, radiation era (PRS friction
    alpha = 3, a ~ tau, tau0 = 1)."""
    from axions_gb300.params import ENERGY_EVOLUTION, MODEL_MOORE, make_params
    return make_params(MODEL_MOORE, n=n, d=0.5, dt=0.1, lam=2.0, lambda2=2.0, lambda12=0.0, eta=1.0, eta2=1.0,
                       q1=1.0, q2=2.0, g=1.0, damped_nt=0, dampFac=0.0, alpha=3.0, scaling=1.0, tau0=1.0,
                       energy_form=ENERGY_EVOLUTION, precision=lat_precision(precision))


def global_string_params(n: int, precision: str):
    """The reference's default physics (mpi_evolution.cpp:15-60): global strings
    (e = 0), lambda = 1, eta = 1, dx = 0.25, dt = 0.05, a damping phase of 200
    steps (0.5), then radiation-era friction (alpha = 3, a ~ tau, tau0 = 1),
    periodic.  (Without damping or friction a random-phase start in a periodic
    box keeps its gradient energy and no network forms.)"""
    from axions_gb300.params import ENERGY_EVOLUTION, F32, F64, make_params
    prec = lat_precision(precision)
    return make_params(0, n=n, d=0.25, dt=0.05, lam=1.0, eta=1.0, g=0.0, damped_nt=200, dampFac=0.5, alpha=3.0,
                       scaling=1.0, tau0=1.0, energy_form=ENERGY_EVOLUTION, precision=prec)


GLOBAL_STRINGS = "e=0, lambda=1, eta=1, dx=0.25, dt=0.05, damped 200 steps (0.5), then alpha=3 friction"


def workload_name(n: int) -> str:
    if MODEL["name"] == "moore":
        return (f"Moore model {n}^3 periodic, phi1/phi2 charges 1/2, eta=1, lambda1=lambda2=2, e=1, dx=0.5, "
                f"dt=0.1, PRS friction alpha=3 (a~tau, tau0=1), independent phases, energy+Gauss every "
                f"{DIAG_EVERY} steps")
    return (f"Abelian-Higgs {n}^3 periodic, lambda=2, e=1, eta=1, dx=0.5, dt=0.1, PRS friction alpha=3 "
            f"(a~tau, tau0=1), energy+Gauss every {DIAG_EVERY} steps")


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# distributed helpers (replicas)
# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws: int, backend: str):
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend=backend)


def dist_barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(ws: int, x: float, device=None) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(ws: int, x: float, device=None) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU implementation (the oracle's restatement of the reference arithmetic)
# ---------------------------------------------------------------------------
def cpu_rate(n: int, seconds: float, min_steps: int = 2, warmup: int = 1):
    """Site-updates/s of the CPU implementation (the oracle's restatement of
    the reference's arithmetic) on all host cores, on the n^3 workload: one
    IC, `warmup` untimed steps, then timed steps (energy/Gauss on every 20th,
    as the workload) until at least `min_steps` steps and `seconds` seconds."""
    from oracle import oracle as O
    p = workload_params(n, "f64_strict")
    st = O.random_phase_ic(p, 42)
    for q in range(max(warmup, 0)):
        O.step(p, st, q, diag=q % DIAG_EVERY == 0)
    steps, t0 = 0, time.perf_counter()
    while True:
        n_step = max(warmup, 0) + steps
        O.step(p, st, n_step, diag=n_step % DIAG_EVERY == 0)
        steps += 1
        el = time.perf_counter() - t0
        if steps >= min_steps and el >= seconds:
            break
    return p.N * steps / el, O.get_threads(), steps, el


# ---------------------------------------------------------------------------
# GPU measurement
# ---------------------------------------------------------------------------
def load_traffic(precision: str, n: int):
    """DRAM traffic per launch of the step kernel from the committed ncu summary."""
    f = ROOT / "profiles" / "traffic.json"
    if not f.exists():
        return None
    try:
        d = json.loads(f.read_text())
        e = d.get(f"{MODEL['name']}_step_{precision}")
        if not e:
            return None
        return e["bytes_per_site"] * n ** 3
    except Exception:
        return None


def fp64_ceiling(precision: str, res: dict, peaks: dict):
    """The second ceiling of an FP64 step: FP64 instructions (DFMA, DADD,
    DMUL per site, from the committed ncu summary) per second against the FP64
    pipe's issue peak, 2 per SM per cycle at the SM clock sampled during the
    timed region."""
    f = ROOT / "profiles" / "traffic.json"
    if precision == "f32" or not f.exists():
        return None
    try:
        d = json.loads(f.read_text())
        e = d.get(f"{MODEL['name']}_step_{precision}")
        if not e or "fp64_inst_per_site" not in e:
            return None
        import torch
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        mhz = (res.get("clocks") or {}).get("sm_mhz") or peaks.get("sm_max_mhz") or 2070.0
        peak = d["fp64_issue_peak_per_sm_per_cycle"] * sms * mhz * 1e6 / 1e9
        ach = e["fp64_inst_per_site"] * res["sites"] / (res["kern_ms"] * 1e-3) / 1e9
        return {"bound": "fp64_pipe", "achieved": ach, "peak": peak, "unit": "G FP64-inst/s", "frac": ach / peak,
                "inst_per_site": e["fp64_inst_per_site"], "sm_mhz": mhz, "sms": sms}
    except Exception:
        return None


def measure_gpu(n: int, precision: str, steps: int, warmup: int, ws: int, local: int, peaks: dict,
                device_ic: bool = False):
    """K steps of the workload with the state resident (CUDA events on the
    library's stream), then the same K steps end to end through lat_run from
    pinned host buffers.  The IC is the host mt19937 one (mpi_evolution.cpp:
    287-312), or with device_ic the device Philox one (for the 768^3 Moore
    lattice, whose host draws would take longer than its steps)."""
    import numpy as np
    import torch

    from axions_gb300 import lattice

    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    p = workload_params(n, precision)
    moore = MODEL["name"] == "moore"
    lat = lattice.Lattice(p)
    lat.set_stream(stream.cuda_stream)
    nc, N = lat.ncomp, lat.N
    pin_now = torch.empty((nc, N), dtype=torch.float64, pin_memory=True)
    if device_ic:
        lat.random_phase_ic_device(42 + local, independent=moore)
        pin_past = torch.empty((nc, N), dtype=torch.float64, pin_memory=True)
        lat.get_state(pin_now.numpy(), pin_past.numpy())
        del pin_past
    else:
        pin_now.numpy()[:] = lattice.random_phase_ic(p, 42 + local, independent=moore)
        lat.set_state(pin_now.numpy(), None, 0)
    ic = pin_now.numpy()

    def one_step():
        return lat.advance(1, DIAG_EVERY)

    for _ in range(warmup):
        one_step()
    torch.cuda.synchronize(dev)
    dist_barrier(ws)
    torch.cuda.synchronize(dev)

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kinds = []
    clock = ClockSampler(local)
    clock.start()
    launches0 = lat.kernel_launches
    t_start.record(stream)
    for q in range(steps):
        nstep = lat.time_step
        kinds.append("diag" if nstep % DIAG_EVERY == 0 else ("store" if (nstep + 1) % DIAG_EVERY == 0 else "plain"))
        evs[q][0].record(stream)
        one_step()
        evs[q][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize(dev)
    launches = lat.kernel_launches - launches0
    dist_barrier(ws)
    torch.cuda.synchronize(dev)
    clocks = clock.stop()
    total_ms = t_start.elapsed_time(t_end)
    per = [a.elapsed_time(b) for a, b in evs]
    plain = [t for t, k in zip(per, kinds) if k == "plain"] or per
    kern_ms = statistics.median(plain)

    # end to end through the C ABI with host buffers (pinned): one lat_run call
    # from the IC, a stationary start whose two levels are one array, as the
    # reference's IC (mpi_evolution.cpp:155-162), to the final level, what the
    # reference's programs write at the end (finalField, ic_w_evolution.cpp:
    # 1183-1187)
    # The host link's rate varies from outside the process (the same pinned
    # upload measured 210 and 45 GB/s in one process), so the run is made
    # E2E_RUNS times and the median reported, with every run's time.
    out_now = torch.empty((nc, N), dtype=torch.float64, pin_memory=True)
    e2e_runs = []
    for _ in range(E2E_RUNS):
        dist_barrier(ws)
        torch.cuda.synchronize(dev)
        e0 = time.perf_counter()
        e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e_start.record(stream)
        diags, _, _ = lat.run(pin_now.numpy(), None, 0, steps, DIAG_EVERY, now_out=out_now.numpy(), past_level=False)
        e_end.record(stream)
        torch.cuda.synchronize(dev)
        e2e_wall = time.perf_counter() - e0
        e2e_runs.append(max(e_start.elapsed_time(e_end), 1e3 * e2e_wall))
        if not np.isfinite(out_now.numpy()).all():
            raise RuntimeError("non-finite field after the end-to-end run")
    lat.close()
    del pin_now, out_now

    level_bytes = nc * N * 8
    return {
        "total_ms": total_ms, "kern_ms": kern_ms, "per_ms": per, "kinds": kinds, "launches": launches,
        "clocks": clocks, "e2e_ms": statistics.median(e2e_runs), "e2e_runs_ms": e2e_runs, "e2e_h2d": level_bytes / steps,
        "e2e_d2h": (level_bytes + 16 * len(diags)) / steps, "sites": N,
    }


def ensemble_jobs(njobs: int, n: int):
    """The batched-ensemble workload: AH n^3 lattices, FP32 fields, each with
    its own seed, lambda ~ U[0.5, 4] and e ~ U[0.5, 2] from a fixed meta-seed."""
    import numpy as np

    from axions_gb300.params import ENERGY_EVOLUTION, F32, make_params
    rng = np.random.default_rng(20260)
    jobs = []
    for q in range(njobs):
        lam = float(rng.uniform(0.5, 4.0))
        e = float(rng.uniform(0.5, 2.0))
        p = make_params(0, n=n, d=0.5, dt=0.1, lam=lam, eta=1.0, g=e, damped_nt=0, dampFac=0.0, alpha=0.0,
                        energy_form=ENERGY_EVOLUTION, precision=F32)
        jobs.append((p, q))
    return jobs


def measure_ensemble(njobs: int, n: int, steps: int, diag_every: int, tick: int, extras: bool = True):
    """Runs/hour of an ensemble: batched (all lattices in the same launches,
    one CUDA graph per tick) against the same jobs run one after another
    through the single-lattice path, in the same FP32 form and (sampled) in
    the plain FP64 form.  Each is timed twice: stepping only (state resident)
    and end to end (IC generation, stepping, diagnostics, download of the
    final fields into a pinned host pair reused by every job)."""
    import numpy as np
    import torch

    from axions_gb300 import lattice
    jobs = ensemble_jobs(njobs, n)
    out = {"jobs": njobs, "lattice": n, "steps": steps, "diag_every": diag_every, "tick_steps": tick,
           "ic": "device Philox-4x32-10 random phases (lat_random_phase_ic_device)"}
    with lattice.Lattice(jobs[0][0]) as tl:   # tune the shape once; new handles start tuned
        tuning = tl.autotune(3)
        nc, N = tl.ncomp, tl.N
    out["tuned_chunk"] = tuning.chunk
    # every job's final fields are downloaded into the same pinned host pair,
    # allocated once, as a driver running an ensemble would do
    pin = [torch.empty((nc, N), dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]

    def run_sequential():
        t_step = 0.0
        t0 = time.perf_counter()
        for p, seed in jobs:
            lat = lattice.Lattice(p)
            lat.random_phase_ic_device(seed)
            torch.cuda.synchronize()
            s0 = time.perf_counter()
            lat.advance(steps, diag_every)
            t_step += time.perf_counter() - s0
            lat.get_state(*pin)
            lat.close()
        return time.perf_counter() - t0, t_step

    def run_batched():
        t0 = time.perf_counter()
        lats = []
        for p, seed in jobs:
            lat = lattice.Lattice(p)
            lat.random_phase_ic_device(seed)
            lats.append(lat)
        torch.cuda.synchronize()
        with lattice.Batch(max(njobs, 1)) as b:
            for lat in lats:
                b.add(lat, diag_every=diag_every, stop_step=steps)
            s0 = time.perf_counter()
            while b.advance(tick) > 0:
                pass
            t_step = time.perf_counter() - s0
            launches = b.kernel_launches
            for lat in lats:
                b.take_diags(lat)
        for lat in lats:
            lat.get_state(*pin)
            lat.close()
        return time.perf_counter() - t0, t_step, launches

    run_batched()      # warm-up: graph capture, module loading
    seq_total, seq_step = run_sequential()
    bat_total, bat_step, launches = run_batched()
    su = njobs * n ** 3 * steps
    out.update({
        "batched": {"runs_per_hour": njobs / bat_step * 3600, "runs_per_hour_e2e": njobs / bat_total * 3600,
                    "site_updates_per_s": su / bat_step, "kernel_launches": launches},
        "sequential": {"runs_per_hour": njobs / seq_step * 3600, "runs_per_hour_e2e": njobs / seq_total * 3600,
                       "site_updates_per_s": su / seq_step},
    })
    # like for like: the batch against the same FP32 jobs run one after another
    out["speedup"] = out["batched"]["runs_per_hour"] / out["sequential"]["runs_per_hour"]
    out["speedup_e2e"] = out["batched"]["runs_per_hour_e2e"] / out["sequential"]["runs_per_hour_e2e"]
    if not extras:
        return out
    # The same jobs run one after another through the plain FP64 path (the
    # form the FP32/batched forms are built beside), sampled on two jobs: a
    # precision comparison, not a batching one.
    t_step = t_total = 0.0
    sampled = jobs[:2]
    for p, seed in sampled:
        q = p.copy()
        q.precision = lat_precision("f64")
        t0 = time.perf_counter()
        lat = lattice.Lattice(q)
        lat.random_phase_ic_device(seed)
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        lat.advance(steps, diag_every)
        t_step += time.perf_counter() - s0
        lat.get_state(*pin)
        lat.close()
        t_total += time.perf_counter() - t0
    if sampled:
        k = len(sampled)
        out["sequential_plain_f64"] = {"runs_per_hour": k / t_step * 3600, "runs_per_hour_e2e": k / t_total * 3600,
                                       "sampled_runs": k, "precision": "f64, the plain two-pass path"}
        out["speedup_vs_plain_f64"] = out["batched"]["runs_per_hour"] / out["sequential_plain_f64"]["runs_per_hour"]
        out["speedup_vs_plain_f64_e2e"] = (out["batched"]["runs_per_hour_e2e"]
                                           / out["sequential_plain_f64"]["runs_per_hour_e2e"])
    # The reference's own way to run an ensemble: one program invocation per
    # job (run_mpi_evol.sh, submit_job.sh).  Timed with the drop-in program on
    # a few jobs; each invocation creates its CUDA context, draws its mt19937
    # IC, steps and exits.
    prog = ROOT / "axions_gb300" / "bin" / "mpi_evolution"
    if prog.exists():
        import subprocess as sp
        import tempfile as tf
        times = []
        for p, seed in jobs[:3]:
            with tf.TemporaryDirectory() as d:
                cmd = [str(prog), f"out_dir={d}", f"nx={n}", f"ny={n}", f"nz={n}", f"nt={steps}", "dx=0.5", "dy=0.5",
                       "dz=0.5", "dt=0.1", f"lambda={p.lam}", f"g={p.g}", "damped_nt=0", "alpha=0", "precision=f32",
                       "stringDetect=false", "calcEnergy=false", f"seed={seed}", "countRate=1000000"]
                t0 = time.perf_counter()
                r = sp.run(cmd, stdout=sp.DEVNULL, stderr=sp.PIPE)
                times.append(time.perf_counter() - t0)
                if r.returncode != 0:
                    times = []
                    break
        if times:
            per = sum(times) / len(times)
            out["program_launches"] = {"seconds_per_run": per, "runs_per_hour": 3600 / per, "sampled_runs": len(times),
                                       "program": "axions_gb300/bin/mpi_evolution precision=f32 (one process per job)"}
            out["speedup_vs_program_launches_e2e"] = out["batched"]["runs_per_hour_e2e"] / (3600 / per)
    del np
    return out


def fp32_vs_fp64(params_fn, n: int, steps: int, diag_every: int, seed: int, independent: bool, check_every: int):
    """One config run twice from the same initial values: FP32 fields with
    FP64 reductions, and the plain FP64 path (parity-tested against the
    oracle).  The IC is the FP32 device IC of `seed` (so both start from the
    same, float-representable values).  Returns the field L2 drift at the end,
    the largest relative energy and Gauss differences over the diagnostic
    steps, and every `check_every` steps the crossing counts and winding
    totals of each scalar."""
    import numpy as np

    from axions_gb300 import lattice
    p32 = params_fn(n, "f32")
    nf = 2 if p32.model == 1 else 1
    ic = None
    runs = {}
    for form in ("f32", "f64"):
        p = params_fn(n, form)
        with lattice.Lattice(p) as lat:
            if ic is None:
                lat.random_phase_ic_device(seed, independent=independent)
                ic = lat.get_state()[0]
            else:
                lat.set_state(ic, None, 0)
            diags, checks = [], []
            t0 = time.perf_counter()
            while lat.time_step < steps:
                k = min(check_every, steps - lat.time_step)
                diags += lat.advance(k, diag_every)
                checks.append({"step": lat.time_step,
                               "crossings": [lat.count_crossings(f) for f in range(nf)],
                               "winding_abs": [lat.winding(f, want_array=False)[1] for f in range(nf)]})
            secs = time.perf_counter() - t0
            now, _ = lat.get_state()
        runs[form] = (np.array([d[1] for d in diags]), np.array([d[2] for d in diags]), now, checks, secs)
    e64, g64, f64, c64, s64 = runs["f64"]
    e32, g32, f32, c32, s32 = runs["f32"]

    def rel(a, b):
        """largest |a-b|/|b| over entries with b != 0 (the Gauss residual of the
        first level is exactly 0)"""
        m = np.abs(b) > 0
        return float(np.max(np.abs(a - b)[m] / np.abs(b)[m])) if m.any() else 0.0

    ns = 2 * nf
    return {
        "lattice": n, "steps": steps, "diag_every": diag_every,
        "field_l2_drift": float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64)),
        "scalar_l2_drift": float(np.linalg.norm(f32[:ns] - f64[:ns]) / np.linalg.norm(f64[:ns])),
        "energy_rel_max": rel(e32, e64), "energy_rel_final": float(abs(e32[-1] - e64[-1]) / abs(e64[-1])),
        "gauss_rel_max": rel(g32, g64), "gauss_rel_final": float(abs(g32[-1] - g64[-1]) / abs(g64[-1])),
        "checks_f64": c64, "checks_f32": c32, "f64_s": s64, "f32_s": s32,
        "speedup_f32": s64 / s32,
    }


def measure_fp32_accuracy(n: int, steps: int, moore_n: int, moore_steps: int):
    """FP32 forms against the FP64 path, per config.
    Config 2 (Abelian-Higgs n^3, radiation era, diagnostics every 20) and
    config 3's physics (Moore, charges 1 and 2, radiation era, both scalars'
    crossings every 50 steps; at moore_n^3, the largest lattice whose FP64 run
    fits the benchmark's time): field L2 drift, energy and Gauss residual, and
    crossing counts and winding totals.  With e != 0 the gauge links drift and
    the reference's detection, which reads phi alone, finds crossings at almost
    every site after a few hundred steps, so a greedy-chained string length of
    these fields is not meaningful (and would chain ~10^8 crossings of one
    percolating cluster); the total string length is compared on global
    strings (the reference's default physics, 128^3, 1000 steps): every 250
    steps L0 + L1 by greedy chaining (ic_w_evolution.cpp:961-1087) and the
    number of crossings."""
    import numpy as np

    from axions_gb300 import lattice
    out = {"config2": fp32_vs_fp64(workload_params, n, steps, DIAG_EVERY, 2026, False, 250)}
    out["config2"]["string_length"] = "not meaningful at e != 0 (about one crossing per site); see global_strings"
    out["config3"] = fp32_vs_fp64(moore_params, moore_n, moore_steps, 50, 2027, True, 500)
    out["config3"]["string_length"] = "not meaningful at e != 0 (about one crossing per site); see global_strings"
    out["config3"]["note"] = f"config 3 physics at {moore_n}^3 (the configured 768^3 x 1500 FP64 run takes ~10 min)"
    gn, gsteps, gevery = 128, 1000, 250
    lens = {}
    for prec in ("f64", "f32"):
        p = global_string_params(gn, prec)
        with lattice.Lattice(p) as lat:
            lat.random_phase_ic_device(2026)
            L, M = [], []
            for s0 in range(0, gsteps, gevery):
                lat.advance(gevery)
                L0, L1, m = lat.string_length(0, True)
                L.append(L0 + L1)
                M.append(m)
        lens[prec] = (np.array(L), np.array(M))
    l64, c64 = lens["f64"]
    l32, c32 = lens["f32"]
    m = l64 > 0
    out["global_strings"] = {
        "physics": GLOBAL_STRINGS, "lattice": gn, "steps": gsteps,
        "every": gevery,
        "string_length_f64": l64.tolist(), "string_length_f32": l32.tolist(),
        "string_length_rel_max": float(np.max(np.abs(l32 - l64)[m] / l64[m])) if m.any() else 0.0,
        "crossings_f64": c64.tolist(), "crossings_f32": c32.tolist()}
    return out


def measure_string_ic(n: int, cpu_n: int):
    """The string initial conditions of initialConditions.cpp at its default
    n^3 = 401^3 lattice (dx 0.5, dt 0.05; g = 1 so the links are not zero):
    the straight-string profile relaxed by bin/singleSemiAnalytic (2001 points
    at h = 0.1: out to r = 200 like the reference's 20001 points at h = 0.01;
    the loop collision's farthest rest-frame distances lie beyond it, as with
    the reference's table), then the
    boosted string (both levels) and the loop collision (both levels, six
    launches) built on the GPU from it (wall time, fields resident, best of
    3).  CPU: the oracle's restatement of the same families (one thread, as
    the reference's serial passes) timed on a cpu_n^3 lattice and scaled by
    the sites."""
    import subprocess as sp
    import tempfile as tf

    import numpy as np
    import torch

    from axions_gb300 import lattice
    from axions_gb300.params import make_params
    from oracle import oracle as O
    prog = ROOT / "axions_gb300" / "bin" / "singleSemiAnalytic"
    with tf.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        r = sp.run([str(prog), f"out_dir={d}", "nx=2001", "h=0.1", "g=1", "digits=17"], stdout=sp.PIPE, stderr=sp.PIPE)
        sor_s = time.perf_counter() - t0
        if r.returncode != 0:
            return {"error": r.stderr.decode()[-200:]}
        prof = np.array([float(t) for t in (Path(d) / "Data" / "SOR_Fields.txt").read_text().split()]).reshape(-1, 2).T
    prof = np.ascontiguousarray(prof)
    h = 0.1
    v = (0.24, 0.5499090833947008, 0.0)
    out = {"lattice": n, "profile": {"program": "bin/singleSemiAnalytic nx=2001 h=0.1 g=1", "seconds": sor_s}}
    p = make_params(0, n=n, d=0.5, dt=0.05, g=1.0)
    with lattice.Lattice(p) as lat:
        for kind in ("boost", "loop_collision"):
            def build():
                if kind == "boost":
                    return lat.boost_ic_device(prof[0], prof[1], h, v)
                return lat.loop_collision_ic_device(prof[0], prof[1], h)
            off = build()
            torch.cuda.synchronize()
            best = 1e30
            for _ in range(3):
                t0 = time.perf_counter()
                build()
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t0)
            pc = make_params(0, n=cpu_n, d=0.5, dt=0.05, g=1.0)
            t0 = time.perf_counter()
            if kind == "boost":
                O.boost_ic(pc, prof[0], prof[1], h, v)
            else:
                from axions_gb300.params import default_loop_collision
                O.loop_collision_ic(pc, prof[0], prof[1], h, default_loop_collision(cpu_n, cpu_n, cpu_n, 0.5, 0.5, 0.5))
            cpu = (time.perf_counter() - t0) * (n / cpu_n) ** 3
            out[kind] = {"gpu_s": best, "sites_per_s": n ** 3 / best, "off_table": off,
                         "cpu_port_s_extrapolated": cpu, "cpu_sample": f"{cpu_n}^3, one thread",
                         "speedup_vs_cpu": cpu / best}
    return out


def measure_string_length(n: int, max_steps: int, max_crossings: int, cpu_sample: int):
    """Total string length by greedy chaining (ic_w_evolution.cpp:961-1087) of
    the crossings of an n^3 lattice of global strings (the reference's default
    physics),
    evolved in FP32 from a random-phase IC in blocks of 250 steps until at most
    `max_crossings` crossings remain (the network has formed; early fields are
    noise whose crossings form one percolating cluster that the greedy rule can
    only walk one crossing at a time) or `max_steps` are done.  GPU: wall time of
    lat_string_length (detection and chaining on the device, link-graph
    component walks).  CPU: the O(M^2) restatement of the reference's loop (one
    thread) timed on the first `cpu_sample` crossings of the same list and
    scaled by (M / sample)^2 to the full list; the GPU chaining of that sample
    is checked against it bit for bit."""
    from axions_gb300 import lattice
    from oracle import oracle as O
    p = global_string_params(n, "f32")
    with lattice.Lattice(p) as lat:
        lat.random_phase_ic_device(2027)
        steps = 0
        while steps < max_steps:
            lat.advance(250)
            steps += 250
            if lat.count_crossings(0) <= max_crossings:
                break
        lat.string_length(0, True)  # buffers
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            L0, L1, M = lat.string_length(0, True)
            times.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        xyz = lat.detect(0)
        t_detect = time.perf_counter() - t0
    sample = xyz[:cpu_sample]
    t0 = time.perf_counter()
    c = O.string_length(p, sample, True)
    t_cpu = time.perf_counter() - t0
    g = lattice.string_length_points(p, sample, True)
    t_gpu = min(times)
    t_ref = t_cpu * (M / max(len(sample), 1)) ** 2
    return {"lattice": n, "steps": steps, "physics": GLOBAL_STRINGS,
            "crossings": M, "L0": L0, "L1": L1, "method": "link-graph component walks",
            "gpu_s": t_gpu, "gpu_crossings_per_s": M / t_gpu, "detect_to_host_s": t_detect,
            "cpu_sample_crossings": len(sample), "cpu_sample_s": t_cpu, "cpu_kind": "port", "cpu_cores": 1,
            "cpu_full_s_extrapolated": t_ref, "speedup_vs_cpu_extrapolated": t_ref / t_gpu,
            "sample_bit_exact": g == c}


def measure_serving(njobs: int, rate: float, budget_gb: float, tick: int, seed: int = 4242):
    """Serving loop under a Poisson stream of jobs: 70 % Abelian-Higgs, 30 %
    Moore, sides from {64, 96, 128, 192, 256}, 200-1000 steps, lambda in
    [0.5, 4], e in [0.5, 2], FP32 fields with FP64 diagnostics every 20 steps,
    device random-phase ICs.  Reports p50/p99 job latency (completion minus
    submission) and the aggregate site-updates/s over the whole run."""
    import threading

    import numpy as np

    from axions_gb300 import lattice
    from axions_gb300.params import ENERGY_EVOLUTION, F32, MODEL_MOORE, make_params
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(njobs):
        n = int(rng.choice([64, 96, 128, 192, 256]))
        steps = int(rng.integers(200, 1001))
        lam, e = float(rng.uniform(0.5, 4.0)), float(rng.uniform(0.5, 2.0))
        if rng.random() < 0.7:
            p = make_params(0, n=n, d=0.5, dt=0.1, lam=lam, eta=1.0, g=e, damped_nt=0, alpha=0.0,
                            energy_form=ENERGY_EVOLUTION, precision=F32)
        else:
            p = make_params(MODEL_MOORE, n=n, d=0.5, dt=0.1, lam=lam, lambda2=lam, eta=1.0, eta2=1.0, q1=1.0, q2=2.0,
                            g=e, damped_nt=0, alpha=0.0, energy_form=ENERGY_EVOLUTION, precision=F32)
        specs.append((p, k, steps, float(rng.exponential(1.0 / rate))))
    ids = []
    with lattice.Server(int(budget_gb * (1 << 30)), tick_steps=tick, max_running=128) as srv:
        def client():
            for p, k, steps, gap in specs:
                time.sleep(gap)
                ids.append(srv.submit(p, seed=k, nsteps=steps, diag_every=20, independent=True))
        th = threading.Thread(target=client)
        th.start()
        th.join()
        res = [srv.wait(i, 3600) for i in ids]
        st = srv.stats()
    ok = [r for r in res if r.status == 2]
    lat_s = np.array([r.end_s - r.submit_s for r in ok])
    span = max(r.end_s for r in ok) - min(r.submit_s for r in res)
    su = sum(r.site_updates for r in ok)
    return {"jobs": njobs, "done": len(ok), "rate_jobs_per_s": rate, "mix": "70% AH / 30% Moore",
            "sides": [64, 96, 128, 192, 256], "steps": "200-1000", "precision": "f32 fields, f64 diagnostics",
            "tick_steps": tick, "hbm_budget_gb": budget_gb,
            "latency_p50_s": float(np.percentile(lat_s, 50)), "latency_p99_s": float(np.percentile(lat_s, 99)),
            "latency_max_s": float(lat_s.max()), "site_updates_per_s": su / span, "makespan_s": span,
            "gpu_busy_frac": st.busy_s / st.wall_s, "peak_hbm_gb": st.peak_bytes / (1 << 30)}


def bench_config(n: int, precision: str, ws: int) -> dict:
    """The `config` of the JSON line, the same for both arms."""
    return {"workload": workload_name(n), "model": "moore" if MODEL["name"] == "moore" else "abelian-higgs",
            "lattice": n, "precision": precision, "diag_every": DIAG_EVERY,
            "l2": f"inputs larger than L2 ({2 * BYTES[MODEL['name']]['f64'] / 3 * n ** 3 / 1e9:.1f} GB FP64 state)",
            "parallelism": "replicas" if ws > 1 else "single"}


def form_entry(res: dict, form: str, n: int, units: float, t_ms: float, steps: int, hbm: float, peaks: dict,
               head_ms: float | None) -> dict:
    ach = bytes_per_site(form) * res["sites"] / (res["kern_ms"] * 1e-3) / 1e9
    e = {"value": units / (t_ms * 1e-3), "ms_per_step": t_ms / steps, "dtype": "f32" if form == "f32" else "f64",
         "kernel_ms": res["kern_ms"], "kernel": kernel_name(form),
         "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                      "traffic": load_traffic(form, n), "bytes_per_site": bytes_per_site(form),
                      "fp64_pipe": fp64_ceiling(form, res, peaks)},
         "e2e": {"value": units / (res["e2e_ms"] * 1e-3), "unit": "site-updates/s",
                 "h2d_bytes_per_step": res["e2e_h2d"], "d2h_bytes_per_step": res["e2e_d2h"],
                 "runs_ms": res["e2e_runs_ms"]},
         "clocks": res["clocks"], "gpu_launches": res["launches"]}
    if head_ms:
        e["speedup_vs_headline"] = head_ms / res["total_ms"]
    return e


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--model", choices=["ah", "moore"], default="ah",
                    help="ah: Abelian-Higgs 512^3 (headline); moore: Moore model 768^3 as the headline")
    ap.add_argument("--n", type=int, default=None, help="lattice side (default 512 for ah, 768 for moore)")
    ap.add_argument("--cpu-n", type=int, default=None, help="side of the CPU lattice (default: the workload's)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--precision", choices=list(FORMS), default="f64",
                    help="form of the headline number (the workload's plain path is f64)")
    ap.add_argument("--no-forms", "--no-fp32", action="store_true", help="measure only the headline form")
    ap.add_argument("--no-moore", action="store_true", help="skip the Moore 768^3 FP32 form (config 3)")
    ap.add_argument("--moore-n", type=int, default=768)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--ensemble-jobs", type=int, default=64)
    ap.add_argument("--ensemble-n", type=int, default=128)
    ap.add_argument("--ensemble-steps", type=int, default=500)
    ap.add_argument("--ensemble-small", type=str, default="64,32", help="further ensemble sides (like for like only)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--serving-jobs", type=int, default=120,
                    help="jobs in the Poisson stream (a sample of the configured 2000)")
    ap.add_argument("--serving-rate", type=float, default=4.0, help="mean arrivals per second")
    ap.add_argument("--serving-saturated-jobs", type=int, default=240,
                    help="jobs of a second stream arriving faster than the GPU serves them (0: skip)")
    ap.add_argument("--serving-saturated-rate", type=float, default=60.0)
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP32-vs-FP64 accuracy study")
    ap.add_argument("--accuracy-n", type=int, default=512, help="lattice side of config 2's accuracy run")
    ap.add_argument("--accuracy-steps", type=int, default=1000)
    ap.add_argument("--accuracy-moore-n", type=int, default=256, help="lattice side of config 3's accuracy run")
    ap.add_argument("--accuracy-moore-steps", type=int, default=1500)
    ap.add_argument("--no-length", action="store_true", help="skip the string-length measurement")
    ap.add_argument("--no-ic", action="store_true", help="skip the string initial-condition measurement")
    ap.add_argument("--ic-n", type=int, default=401)
    ap.add_argument("--length-n", type=int, default=512)
    ap.add_argument("--length-max-steps", type=int, default=4000)
    ap.add_argument("--length-max-crossings", type=int, default=1500000)
    ap.add_argument("--length-cpu-sample", type=int, default=20000)
    args = ap.parse_args()
    ws, rank, local = dist_env()
    MODEL["name"] = args.model
    n = args.n if args.n else (args.moore_n if args.model == "moore" else 512)
    cpu_n = args.cpu_n or n
    steps, warmup = args.steps, max(args.warmup, 0)

    if args.impl == "reference":
        # the reference's arithmetic on the host cores (the oracle's restatement,
        # pinned bit-exact against reference builds): the same workload, lattice
        # and step count; rank 0 alone under torchrun
        if rank != 0:
            return
        MODEL["name"] = "ah"
        r, cores, ns, el = cpu_rate(cpu_n, 0.0, min_steps=steps, warmup=warmup)
        line = {"impl": "reference", "metric": "site-updates/s", "value": r, "unit": "site-updates/s",
                "n_gpus": args.gpus, "steps": ns, "warmup": warmup, "ms_per_step": 1e3 * el / ns,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic: seeded uniform-phase IC (mt19937, mpi_evolution.cpp:287-312)",
                "config": bench_config(cpu_n, "f64", args.gpus),
                "cpu_baseline": {"value": r, "unit": "site-updates/s", "cores": cores, "kind": "port",
                                 "sample": f"the {cpu_n}^3 workload itself, {ns} steps after {warmup} warm-up "
                                           f"steps, {el:.1f} s"},
                "e2e": {"value": r, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    # CPU baseline before the first CUDA call (rank 0, one GPU only)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu and args.model == "ah":
        r, cores, ns, el = cpu_rate(cpu_n, args.cpu_seconds, warmup=1)
        cpu = {"value": r, "unit": "site-updates/s", "cores": cores, "kind": "port",
               "sample": f"the {cpu_n}^3 workload itself, {ns} steps in {el:.1f} s after 1 warm-up step"}

    t_start = time.perf_counter()
    import torch
    torch.cuda.set_device(local)
    dist_init(ws, "nccl")
    dev = torch.device("cuda", local)
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0

    def note(leg, t0):
        print(f"bench: {leg} done in {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)

    head = args.precision
    dev_ic = args.model == "moore"
    res = measure_gpu(n, head, steps, warmup, ws, local, peaks, device_ic=dev_ic)
    t_max = dist_max(ws, res["total_ms"], dev)
    units = dist_sum(ws, float(res["sites"]) * steps, dev)
    e2e_max = dist_max(ws, res["e2e_ms"], dev)
    forms = {}
    for form in ([] if args.no_forms else [f for f in FORMS if f != head]):
        r2 = measure_gpu(n, form, steps, warmup, ws, local, peaks, device_ic=dev_ic)
        t2 = dist_max(ws, r2["total_ms"], dev)
        r2["e2e_ms"] = dist_max(ws, r2["e2e_ms"], dev)
        forms[form] = form_entry(r2, form, n, units, t2, steps, hbm, peaks, res["total_ms"])
    note("headline and forms", t_start)
    moore = None
    if args.model == "ah" and not args.no_moore:
        t_leg = time.perf_counter()
        MODEL["name"] = "moore"
        rm = measure_gpu(args.moore_n, "f32", steps, warmup, ws, local, peaks, device_ic=True)
        tm = dist_max(ws, rm["total_ms"], dev)
        rm["e2e_ms"] = dist_max(ws, rm["e2e_ms"], dev)
        um = dist_sum(ws, float(rm["sites"]) * steps, dev)
        moore = form_entry(rm, "f32", args.moore_n, um, tm, steps, hbm, peaks, None)
        moore["config"] = bench_config(args.moore_n, "f32", ws)
        moore["data"] = "synthetic: seeded independent uniform phases per scalar (device Philox-4x32-10)"
        MODEL["name"] = "ah"
        note("moore", t_leg)
    t_leg = time.perf_counter()
    ensemble = None
    if not args.no_ensemble:
        ensemble = measure_ensemble(args.ensemble_jobs, args.ensemble_n, args.ensemble_steps, DIAG_EVERY, 50)
        ensemble["smaller"] = {}
        for side in [int(x) for x in args.ensemble_small.split(",") if x.strip()]:
            ensemble["smaller"][str(side)] = measure_ensemble(args.ensemble_jobs, side, args.ensemble_steps,
                                                              DIAG_EVERY, 50, extras=False)
    note("ensemble", t_leg)
    t_leg = time.perf_counter()
    serving = serving_sat = None
    if not args.no_serving:
        serving = measure_serving(args.serving_jobs, args.serving_rate, 96.0, 25)
        serving["note"] = f"a {args.serving_jobs}-job sample of the configured 2000-job stream"
        if args.serving_saturated_jobs > 0:
            serving_sat = measure_serving(args.serving_saturated_jobs, args.serving_saturated_rate, 96.0, 25,
                                          seed=4343)
            serving_sat["note"] = "arrivals faster than the GPU serves them: the engine's own throughput"
    note("serving", t_leg)
    t_leg = time.perf_counter()
    accuracy = None
    if not args.no_accuracy and args.model == "ah":
        accuracy = measure_fp32_accuracy(args.accuracy_n, args.accuracy_steps, args.accuracy_moore_n,
                                         args.accuracy_moore_steps)
    note("accuracy", t_leg)
    t_leg = time.perf_counter()
    slen = None
    if not args.no_length and args.model == "ah" and rank == 0:
        slen = measure_string_length(args.length_n, args.length_max_steps, args.length_max_crossings,
                                     args.length_cpu_sample)
    note("string length", t_leg)
    t_leg = time.perf_counter()
    string_ic = None
    if not args.no_ic and args.model == "ah" and rank == 0:
        string_ic = measure_string_ic(args.ic_n, 48)
    note("string initial conditions", t_leg)
    if rank != 0:
        return
    MODEL["name"] = args.model
    achieved = bytes_per_site(head) * res["sites"] / (res["kern_ms"] * 1e-3) / 1e9
    line = {
        "metric": "site-updates/s", "value": units / (t_max * 1e-3), "unit": "site-updates/s", "n_gpus": ws,
        "steps": steps, "warmup": warmup, "ms_per_step": t_max / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if head == "f32" else "f64",
        "data": "synthetic: seeded uniform-phase IC (mt19937, mpi_evolution.cpp:287-312)",
        "config": bench_config(n, head, ws),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": load_traffic(head, n), "peak_source": peak_src,
                     "kernel": kernel_name(head), "kernel_ms": res["kern_ms"],
                     "bytes_per_site": bytes_per_site(head), "fp64_pipe": fp64_ceiling(head, res, peaks)},
        "cpu_baseline": cpu,
        "e2e": {"value": units / (e2e_max * 1e-3), "unit": "site-updates/s",
                "h2d_bytes_per_step": res["e2e_h2d"], "d2h_bytes_per_step": res["e2e_d2h"],
                "runs_ms": res["e2e_runs_ms"], "statistic": f"median of {E2E_RUNS} runs (max over ranks)"},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
        "forms": forms,
        "moore": moore,
        "ensemble": ensemble,
        "serving": serving,
        "serving_saturated": serving_sat,
        "fp32_accuracy": accuracy,
        "string_length": slen,
        "string_ic": string_ic,
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
