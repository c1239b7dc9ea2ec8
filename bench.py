"""Benchmark: compartment-steps/s of the batched uneven HH cable population.

Workload: 16,384 HH cables with odd compartment counts U[51, 401]
(3.70 M compartments), float32 state, extracellular point-source stimulation
(cathodic 0.1 ms pulse), dt 0.005 ms for 10 ms = 2000 timesteps.  One bench
"step" is one full 2000-timestep run of the whole population: a single
persistent launch of dgb_cable_run.

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  ``value`` is timed with CUDA events on the launching
stream with inputs resident in HBM; ``e2e`` is the same metric through the
public API from pinned host buffers (state + prepared workspace in, spike
results + final voltages out, copies inside the timed region).  The reference
arm (``--impl reference``) times the CPU restatement of the reference's
PyTorch CPU cable solver (oracle port) on all host cores on a bounded sample.
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

METRIC = "compartment-steps/s"
ALG_BYTES_PER_COMP_STEP = 48  # unfused per-step traffic of one float32 compartment-step
# persistent kernel of the 16,384-cable population under ncu (4,096 cables x 100 steps, float32 fast
# math): DRAM bytes per compartment per launch, thread instructions per
# compartment-step (profiles/ holds the capture's summary)
C2_NCU_DRAM_BYTES_PER_COMP = 22536960 / 932014
C2_NCU_THREAD_INSTR_PER_COMP_STEP = 691476115 * 31.55 / 93201400


def _issue_bound(instr_per_unit, units, ms, clocks, dev):
    """The on-chip bound of an issue-bound kernel: the time its instructions
    take at one instruction per scheduler per cycle on every SM at the timed
    region's median SM clock, as a fraction of the measured time."""
    import torch

    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = (clocks.summary() or {}).get("sm_mhz") or 2070.0
    ceiling_ms = instr_per_unit * units / (sms * 4 * 32 * mhz * 1e6) * 1e3
    return {"bound": "issue", "thread_instructions_per_unit": instr_per_unit,
            "ceiling_ms": ceiling_ms, "frac": ceiling_ms / ms, "sm_mhz": mhz,
            "note": "instructions per compartment-step from the ncu capture; ceiling = "
                    "all 4 schedulers of every SM issuing every cycle"}
L2_BYTES = 129 * 1024 * 1024


def eager_reference_step(pop, bands, step):
    """One timestep with the reference's eager structure on the packed population.

    Every elementwise operation of the mechanism advance (mod/HH.py:24-40,
    mechanisms/_cnexp.py:96-132), the current frame (HH.py:109-116) and the
    increment-form assembly (integrators/implicit.py:569-664) is its own torch
    kernel, as in the reference's JIT=0 CUDA path; the solve is one call of the
    ragged tridiagonal kernel with the update v += dv (the reference calls its
    Triton Thomas kernel there).  A measurement baseline only: the product
    path is dgb_cable_run."""
    import torch

    from dendra_gb300 import _lib
    from dendra_gb300.cable import AH1, AM1, AN1, q10_of

    d = pop._dev
    v, m, h, n = pop.v, pop.m, pop.h, pop.n
    q10, dt, dt_s = q10_of(pop.celsius), pop.dt, pop.dt_s

    def vtrap(x):
        q = x / 10.0
        local = q.abs() <= 1.0
        q2 = q * q
        val = q2 * (-691.0 / 1307674368000.0) + 1.0 / 47900160.0
        val = val * q2 - 1.0 / 1209600.0
        val = val * q2 + 1.0 / 30240.0
        val = val * q2 - 1.0 / 720.0
        val = val * q2 + 1.0 / 12.0
        series = (10.0 - x / 2.0) + x * (q * val)
        return torch.where(local, series, x / (torch.exp(q) - 1.0))

    def phi1(z):
        val = z * (1.0 / 3628800.0) + 1.0 / 362880.0
        for c in (40320.0, 5040.0, 720.0, 120.0, 24.0, 6.0, 2.0, 1.0):
            val = val * z + 1.0 / c
        return val

    def cnexp(x, a, b):
        z = -b * dt
        small = z.abs() <= 0.5
        taylor = x + dt * (a - b * x) * phi1(z)
        eq = a / b
        return torch.where(small, taylor, eq + (x - eq) * torch.exp(z))

    am = AM1 * vtrap(-(v + 40.0))
    bm = 4.0 * torch.exp(-(v + 65.0) / 18.0)
    ah = AH1 * torch.exp(-(v + 65.0) / 20.0)
    bh = 1.0 / (torch.exp(-(v + 35.0) / 10.0) + 1.0)
    an = AN1 * vtrap(-(v + 55.0))
    bn = 0.125 * torch.exp(-(v + 65.0) / 80.0)
    m.copy_(cnexp(m, q10 * am, q10 * (am + bm)))
    h.copy_(cnexp(h, q10 * ah, q10 * (ah + bh)))
    n.copy_(cnexp(n, q10 * an, q10 * (an + bn)))
    gna = d["gnabar"] * m * m * m * h
    n2 = n * n
    gk = d["gkbar"] * (n2 * n2)
    G = d["gl"] + gna + gk
    J = d["gl"] * d["el"] + gna * pop.ena + gk * pop.ek
    gr, gl = d["g_right"], d["g_left"]
    v_next = torch.cat([v[1:], v[-1:]])
    v_prev = torch.cat([v[:1], v[:-1]])
    fn = (J - G * v) * d["scale"] + (gr * (v_next - v) - gl * (v - v_prev))
    if "field" in d:
        t = torch.tensor(step * dt, dtype=torch.float64, device=v.device).to(pop.dtype)
        on = (t >= d["ve_delay"]) & (t < d["ve_delay"] + d["ve_pw"])
        amp = torch.where(on, d["ve_amp"], torch.zeros_like(d["ve_amp"]))
        ve = d["field"] * amp[d["comp_cable"].long()]
        ve_next = torch.cat([ve[1:], ve[-1:]])
        ve_prev = torch.cat([ve[:1], ve[:-1]])
        fn = fn + (gr * (ve_next - ve) - gl * (ve - ve_prev))
    torch.mul(fn, dt_s, out=bands[3])
    torch.sub(1.0, dt_s * ((-gr - gl) - G * d["scale"]), out=bands[1])
    torch.mul(gl, -dt_s, out=bands[0])
    torch.mul(gr, -dt_s, out=bands[2])
    args = pop._args(1)
    with torch.cuda.device(v.device):
        rc = _lib.load().dgb_cable_solve_update(args, *(bands[i].data_ptr() for i in range(4)),
                                                _lib.stream_ptr(v.device))
    _lib.check(rc, "dgb_cable_solve_update")


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


COVERED_TIMING = ("CUDA events on the launching stream; a 1 ms device sleep before the "
                  "start event keeps host enqueue out of the events")


def _cover_enqueue():
    """Queue a device sleep (about 1 ms) right before a start event, so
    the stream is still busy while the host enqueues the event and the timed
    launch: the events then bracket the kernel, not host enqueue latency.  The
    sleep runs before the start event and is not timed.  Host overhead is in
    each line's ``e2e`` figure instead."""
    import torch

    torch.cuda._sleep(2_000_000)


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_baseline(n_sample: int, steps: int, threads: int | None = None):
    """Oracle port of the reference CPU cable update on a subsample of the
    16,384-cable population."""
    import torch

    import oracle
    from dendra_gb300.workloads import cable_population_c2

    rng = np.random.default_rng(99)
    subset = np.sort(rng.choice(16384, n_sample, replace=False))
    pop = cable_population_c2(dtype=torch.float32, device="cpu", subset=subset)
    p = pop.problem_dict()
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    t0 = time.perf_counter()
    oracle.cable_run(p, steps)
    dt = time.perf_counter() - t0
    return pop.N * steps / dt, pop.N, dt, oracle.num_threads()


def _c2_samples():
    """Two accuracy samples of the 16,384-cable population: every 128th cable, and the 128 most
    strongly driven cables (largest |amp| / distance; about half of them fire)."""
    from dendra_gb300.workloads import c2_spec

    s = c2_spec()
    drive = np.abs(s["amp"]) / s["dist"]
    return (("every 128th cable", np.arange(0, 16384, 128)),
            ("128 most strongly driven cables", np.sort(np.argsort(-drive)[:128])))


def _c2_gpu_outputs(dev, fast_math, steps=2000, every=10):
    """The float32 GPU run of each accuracy sample: traces of every compartment
    every `every` steps and the crossings at both ends and the middle."""
    from dendra_gb300.workloads import cable_population_c2

    outs = []
    for name, sub in _c2_samples():
        pop = cable_population_c2(device=dev, subset=sub, fast_math=fast_math)
        idx = np.array([[0, k // 2, k - 1] for k in pop.n_comp], dtype=np.int32)
        import torch

        r = pop.run(steps, rec_every=every, record_all=True, raster=torch.as_tensor(idx),
                    raster_cap=64)
        outs.append((name, sub, idx, r.trace_all.double().cpu().numpy(),
                     r.raster.count.cpu().numpy(), r.raster.steps.cpu().numpy()))
    return outs


def _c2_accuracy(gpu_outs, steps=2000, every=10):
    """float32 GPU vs the float64 oracle (float32 pulse grid, same inputs),
    and the reference's own float32 arithmetic (the oracle in float32) beside it."""
    import oracle
    from dendra_gb300.workloads import cable_population_c2

    res = {}
    for name, sub, idx, tr, cnt, stp in gpu_outs:
        pop = cable_population_c2(device="cpu", subset=sub)
        p32 = pop.problem_dict()
        p64 = {k: (v.astype(np.float64) if isinstance(v, np.ndarray) and v.dtype.kind == "f"
                   else v) for k, v in p32.items()}
        _, _, _, _, j = oracle.cable_run(p64, steps, rec_every=every, gate_f32=True,
                                         record_all=True, raster=idx, raster_cap=64)
        _, _, _, _, o32 = oracle.cable_run(pop.problem_dict(), steps, rec_every=every,
                                           record_all=True)
        res[name] = {
            "max_abs_dv_mv": float(np.abs(tr - j["trace_all"]).max()),
            "reference_float32_arithmetic_max_abs_dv_mv":
                float(np.abs(o32["trace_all"].astype(np.float64) - j["trace_all"]).max()),
            "spike_steps_identical": bool(np.array_equal(cnt, j["rast_count"]) and
                                          np.array_equal(stp, j["rast_steps"])),
            "crossings": int(j["rast_count"].sum()),
            "cables_firing": int((j["rast_count"].max(axis=1) > 0).sum())}
    return {"reference": "float64 oracle on the same inputs and float32 pulse grid; every "
                         "compartment every 10 steps over 2000 steps; crossings at both ends "
                         "and the middle", "samples": res}


REF_DIR = os.path.join(ROOT, "baseline", "_ref")
REF_SHIM = os.path.join(ROOT, "tests", "golden", "refshim")
# cables of the 16,384-cable population grouped by compartment count, as the reference needs one
# Unmyelinated population per K; the timed sample is these groups
C2_REF_GROUPS = (51, 225, 401)


def _ref_child(kind, steps, reps, warmup):
    """Runs inside the reference child process (PYTHONPATH = the installed
    reference + its import shims): the reference's own CPU solver path through
    its public API, dn.Unmyelinated + insert(hh) + integrator bwd_euler_ub at
    JIT=0 (pcr_solve_t without dendra-solvers), on all host cores.  Builds the
    models once, runs `warmup` untimed and `reps` timed model.run calls of
    `steps` timesteps each, and prints one JSON object with the
    compartment-steps per call and the wall time of each timed call."""
    import importlib.util
    import types
    import warnings

    import torch

    # networkx is imported by the reference's model modules but used only by
    # its graph and tree front ends, never on the cable path timed here; where
    # the host lacks it, an empty stand-in module satisfies the import
    if importlib.util.find_spec("networkx") is None:
        sys.modules["networkx"] = types.ModuleType("networkx")
    import dendra as dn
    from dendra.models.mod import hh

    warnings.filterwarnings("ignore")
    torch.set_num_threads(os.cpu_count() or 1)
    models, groups = [], []
    device = "cuda" if kind == "c2gpu" else "cpu"
    if kind == "c2gpu":
        kind = "c2"
    with dn.ctx(JIT=0):
        if kind == "c2":
            from dendra_gb300.workloads import RHOE_OHM_CM, c2_spec

            s = c2_spec()
            for K in C2_REF_GROUPS:
                idx = np.nonzero(s["ks"] == K)[0]
                dx = float(np.mean(s["length"][idx] / K))
                model = dn.Unmyelinated([float(d) for d in s["diam"][idx]], L=(K - 1) * dx,
                                        dx=dx, celsius=6.3, v_init=-65.0, dtype=torch.float32,
                                        integrator=dn.bwd_euler_ub(), rhoa=100.0)
                model.insert(hh)
                if device == "cuda":
                    model.to("cuda")
                model.initialize()
                Kr = int(model.v.shape[-1])
                x = (torch.arange(Kr, dtype=torch.float64) - (Kr - 1) / 2) * dx
                r_cm = torch.sqrt(x[None, :] ** 2 +
                                  torch.as_tensor(s["dist"][idx])[:, None] ** 2) * 1e-4
                spatial = (RHOE_OHM_CM / (4 * torch.pi * r_cm)
                           * torch.as_tensor(s["amp"][idx])[:, None]).to(torch.float32)
                spatial = spatial.to(device)
                extra = (spatial, dn.mono_rect(amp=1.0, delay=0.0, pw=0.1))
                models.append((model, 0.005, dict(extra=extra)))
                groups.append([K, int(len(idx)), Kr])
        else:  # c1: 64 x 101 float64 cables, somatic clamp, Recorder(v) of every compartment
            rng = np.random.default_rng(1)
            amp = torch.as_tensor(rng.uniform(0.05, 0.5, 64) * 1e-6).reshape(64, 1)
            model = dn.Unmyelinated([1.0] * 64, L=1000.0, dx=10.0, celsius=6.3, v_init=-65.0,
                                    dtype=torch.float64, integrator=dn.bwd_euler_ub(),
                                    rhoa=100.0)
            model.insert(hh)
            model[..., 0].inject(dn.mono_rect(amp=amp, delay=5.0, pw=1.0))
            model.initialize()
            models.append((model, 0.025, dict(callbacks=[dn.Recorder(("v",))])))
            groups.append([101, 64, int(model.v.shape[-1])])
        units = sum(int(m.v.numel()) for m, _, _ in models) * steps
        times = []
        for rep in range(warmup + reps):
            secs = 0.0
            for model, dt, kw in models:
                model.initialize()
                if device == "cuda":
                    torch.cuda.synchronize()
                t0 = time.perf_counter()
                model.run(dt=dt, duration=steps * dt, **kw)
                if device == "cuda":
                    torch.cuda.synchronize()
                secs += time.perf_counter() - t0
            if rep >= warmup:
                times.append(secs)
    print(json.dumps({"units": units, "times": times, "groups": groups,
                      "threads": torch.get_num_threads(), "cores": os.cpu_count(),
                      "torch": torch.__version__}), flush=True)


def reference_cpu(kind, steps, reps=1, warmup=0, timeout=900):
    """Time the installed reference (baseline/_ref) in a child process; returns
    its JSON dict, or {"error": why} when the reference cannot run here.
    kind "c2gpu" runs the reference's own CUDA path (its Triton Thomas solver
    and eager mechanism kernels); the Triton release on the GPU hosts bundles a
    ptxas that does not know sm_103a, so Triton is pointed at the CUDA
    toolkit's ptxas (TRITON_PTXAS_PATH) when one is installed."""
    if not os.path.isdir(os.path.join(REF_DIR, "dendra")):
        return {"error": "reference not installed in baseline/_ref"}
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([REF_DIR, REF_SHIM, ROOT, env.get("PYTHONPATH", "")])
    ptxas = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "ptxas")
    if kind == "c2gpu" and "TRITON_PTXAS_PATH" not in env and os.path.exists(ptxas):
        env["TRITON_PTXAS_PATH"] = ptxas
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--ref-child", kind,
           "--ref-steps", str(steps), "--steps", str(reps), "--warmup", str(warmup)]
    try:
        r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=timeout)
    except subprocess.TimeoutExpired:
        return {"error": f"reference run exceeded {timeout} s"}
    for line in reversed(r.stdout.splitlines()):
        if line.startswith("{"):
            return json.loads(line)
    tail = (r.stderr or r.stdout).strip().splitlines()[-1:] or ["no output"]
    return {"error": f"reference run failed (rc {r.returncode}): {tail[0][:300]}"}


def reference_baseline(kind, steps, reps=1, warmup=0):
    """cpu_baseline dict of the reference's own CPU path, or None (with the reason)."""
    r = reference_cpu(kind, steps, reps, warmup)
    if "error" in r:
        return None, r["error"]
    secs = float(np.median(r["times"]))
    if kind == "c2":
        n_cab = sum(g[1] for g in r["groups"])
        what = (f"16,384-cable population groups K={list(C2_REF_GROUPS)} ({n_cab} cables "
                "with their own diameters and electrodes, one Unmyelinated population "
                f"per K) x {steps} timesteps, float32")
    else:
        what = f"64 x 101 float64 cables with Recorder(v) for {steps} of their 2000 steps"
    return {"value": r["units"] / secs, "unit": METRIC, "cores": r["threads"],
            "kind": "reference",
            "sample": f"{what}; the reference's model.run at JIT=0 (pcr_solve_t), torch "
                      f"{r['torch']} with {r['threads']} threads", "seconds": secs}, None


def run_reference(args, world, rank):
    """Reference arm of the 16,384-cable population: the reference's own PyTorch CPU solver
    (baseline/_ref, model.run through its public API) on all host cores, on
    three of the population's equal-K groups (their own cables, float32,
    extracellular pulse) for --ref-steps timesteps per bench step.  The C port
    of the same update (oracle) is timed beside it and reported as a second
    figure; it becomes the line's value only when the reference cannot run."""
    if rank != 0:
        return
    cpu, why = reference_baseline("c2", args.ref_steps, args.steps, args.warmup)
    pv, n_comp, psecs, pcores = cpu_baseline(args.sample, 200)
    port = {"value": pv, "unit": METRIC, "cores": pcores, "kind": "port",
            "sample": f"{args.sample} of 16384 cables ({n_comp} compartments) x 200 timesteps, "
                      "float32, the oracle's C restatement"}
    if cpu is None:
        cpu, ms = dict(port, note=why), psecs * 1e3
    else:
        ms = cpu.pop("seconds") * 1e3
    value = cpu["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "c2-uneven-hh-cables-extracellular", "n_cables": 16384,
                   "k_range": [51, 401], "dt_ms": 0.005, "timesteps": 2000},
        "cpu_baseline": cpu, "cpu_port": port,
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _reference_solve_line(args, world, metric, cfg, units, solve, sample):
    """Reference arm of a single-solve workload: the oracle's CPU restatement
    of the reference solver (all host threads it uses), timed with
    perf_counter over ``args.steps`` solves after ``args.warmup`` warm-up
    solves; prints the reference JSON line."""
    import oracle

    for _ in range(args.warmup):
        solve()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        solve()
        times.append(time.perf_counter() - t0)
    secs = float(np.mean(times))
    value = units / secs
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": metric, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": value, "unit": metric, "cores": oracle.num_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": metric, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)

C1_RASTER = (0, 5, -5)  # soma and the reference Raster's default node_check [5, -5]


def _c1_problem():
    """The 64 x 101 float64 population on the host with its raster indices."""
    import torch

    from dendra_gb300.workloads import cable_population_c1

    pop = cable_population_c1(device="cpu", dtype=torch.float64)
    idx = np.array([[c % k for c in C1_RASTER] for k in pop.n_comp], dtype=np.int32)
    return pop, idx


def _c1_oracle(threads=None):
    """The float64 oracle on the full 64-cable run: (seconds, outputs, cores)."""
    import oracle

    pop, idx = _c1_problem()
    p = pop.problem_dict()
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    from dendra_gb300.workloads import C1_STEPS

    t0 = time.perf_counter()
    _, _, _, _, out = oracle.cable_run(p, C1_STEPS, record_all=True, raster=idx, raster_cap=256)
    return time.perf_counter() - t0, out, oracle.num_threads(), pop.N * C1_STEPS


def _apply_launch(pop, launch):
    """--launch for configs 1 and 4: its first field fixes the cables per CTA
    of the persistent runs, -1 the split-gate run (one cable on 4 warps);
    empty keeps the library's default shape."""
    if not launch:
        return
    w = int(launch.split(",")[0])
    pop.split_gates = w < 0
    pop.warps_per_block = max(w, 0)


def bench_c1(args, world, rank, local):
    """64 HH cables x 101 compartments (L 1000 um, dx 10 um, diam 1 um,
    Ra 100 ohm cm), float64, backward Euler + cnexp at dt 0.025 ms for 2000
    steps, a 1 ms somatic clamp at 5 ms of U[0.05, 0.5] nA.  One bench step is
    the whole run with its outputs: the full (2001, 64, 101) voltage trace and
    every 0 mV upward crossing at the soma and at compartments 5 and -5, from
    one persistent launch."""
    cfg = {"workload": "c1-hh-cables-full-traces", "n_cables": 64, "compartments": 101,
           "dt_ms": 0.025, "timesteps": 2000, "state_dtype": "float64",
           "outputs": "full (2001, 64, 101) v trace + every 0 mV upward crossing at "
                      "compartments 0, 5, -5"}
    if args.impl == "reference":
        if rank != 0:
            return
        secs, _, cores, units = _c1_oracle()
        port = {"value": units / secs, "unit": METRIC, "cores": cores, "kind": "port",
                "sample": "the whole 64-cable run (12.9 M compartment-steps, full traces and "
                          "raster), the oracle's C restatement"}
        cpu, why = reference_baseline("c1", args.ref_steps * 5, args.steps, args.warmup)
        if cpu is None:
            cpu, ms = dict(port, note=why), secs * 1e3
        else:
            ms = cpu.pop("seconds") * 1e3
        value = cpu["value"]
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "cpu_baseline": cpu, "cpu_port": port,
                "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    import torch

    import dendra_gb300
    from dendra_gb300.workloads import C1_STEPS, cable_population_c1

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dendra_gb300.load()
    pop = cable_population_c1(device=dev)
    _apply_launch(pop, args.launch)
    state0 = tuple(t.clone() for t in (pop.v, pop.m, pop.h, pop.n))

    def reset():
        for dst, src in zip((pop.v, pop.m, pop.h, pop.n), state0):
            dst.copy_(src)
        pop.step_index, pop.t = 0, 0.0

    def run():
        reset()
        return pop.run(C1_STEPS, record_all=True, raster=list(C1_RASTER), raster_cap=256,
                       spk_thr=0.0)

    for _ in range(max(3, args.warmup)):
        run()
    torch.cuda.synchronize()
    pop.check_status()
    flush = torch.ones(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    times = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.sum()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            res = run()
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    units = pop.N * C1_STEPS
    value = units / (ms * 1e-3)
    trace = res.trace_all.cpu().numpy()
    rast = {k: getattr(res.raster, k).cpu().numpy() for k in ("count", "steps")}

    # end to end through the public API: inputs from pinned host memory, the
    # full trace and the raster back to pinned host memory
    host_in = {k: v.detach().cpu().pin_memory() for k, v in pop._dev.items()}
    host_state = [t.cpu().pin_memory() for t in state0]
    h2d = sum(t.numel() * t.element_size() for t in host_in.values())
    h2d += sum(t.numel() * t.element_size() for t in host_state)
    out_tr = torch.empty(trace.shape, dtype=torch.float64).pin_memory()
    out_cnt = torch.empty(rast["count"].shape, dtype=torch.int32).pin_memory()
    out_steps = torch.empty(rast["steps"].shape, dtype=torch.int64).pin_memory()
    d2h = sum(t.numel() * t.element_size() for t in (out_tr, out_cnt, out_steps))

    def e2e_step():
        for k, t in host_in.items():
            pop._dev[k].copy_(t, non_blocking=True)
        for dst, src in zip((pop.v, pop.m, pop.h, pop.n), host_state):
            dst.copy_(src, non_blocking=True)
        pop.step_index, pop.t = 0, 0.0
        r = pop.run(C1_STEPS, record_all=True, raster=list(C1_RASTER), raster_cap=256,
                    spk_thr=0.0)
        out_tr.copy_(r.trace_all, non_blocking=True)
        out_cnt.copy_(r.raster.count, non_blocking=True)
        out_steps.copy_(r.raster.steps, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    peak, peak_kind = _peaks()
    achieved = 2 * ALG_BYTES_PER_COMP_STEP * units / (ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {**cfg, "l2": "flushed between timed steps (256 MiB read, outside the events)",
                   "launch": "one persistent dgb_cable_run launch per step (trace_all + raster)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "note": (f"{2 * ALG_BYTES_PER_COMP_STEP} algorithmic B per float64 "
                              "compartment-step of the unfused update; 64 cables on 64 CTAs "
                              "of 4 warps (gates split over the SM sub-partitions): bound by "
                              "the FP64 rate of 64 SMs, not by HBM "
                              f"({peak_kind} copy bandwidth)")},
        "e2e": {"value": units / (e2e_ms * 1e-3), "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms},
        "gpu_launches": 2 * args.steps,
        "clocks": clocks.summary(),
        "spikes": {"crossings_soma": int(rast["count"][:, 0].sum()),
                   "cables_firing": int((rast["count"][:, 0] > 0).sum())},
    }
    if rank == 0 and not args.no_cpu:
        secs, ref, cores, _ = _c1_oracle()
        port = {"value": units / secs, "unit": METRIC, "cores": cores, "kind": "port",
                "sample": "the whole 64-cable run, float64 oracle, full traces and raster"}
        cpu, why = reference_baseline("c1", 200)
        if cpu is None:
            cpu = dict(port, note=why)
        else:
            cpu.pop("seconds")
        line["cpu_baseline"] = cpu
        line["cpu_port"] = port
        line["accuracy"] = {
            "max_abs_dv_mv_vs_float64_oracle": float(np.abs(trace - ref["trace_all"]).max()),
            "spike_steps_identical": bool(np.array_equal(rast["count"], ref["rast_count"]) and
                                          np.array_equal(rast["steps"], ref["rast_steps"])),
            "reference": "float64 CPU oracle of the reference update, same inputs"}
    if rank == 0:
        print(json.dumps(line), flush=True)


C3_BYTES_PER_COMP_STEP = 24  # unfused tree step: v r/w 8 B + main/rhs/axial/parent 16 B


def bench_c3(args, world, rank, local):
    """4,096 branched cells (200-2,000 compartments, HH soma, passive
    dendrites), 100 Exp2Syn inputs each from random cells (409,600 NetCons,
    lognormal(-7, 0.5) uS, delays U[1, 5] ms), 5 Hz Poisson background, float32,
    dt 0.025 ms for 200 ms (8,000 steps).  One bench step = the whole run."""
    import torch

    import oracle
    from dendra_gb300.network import random_network

    n_cells = min(args.cables, 4096) if args.cables != 16384 else 4096
    t_stop = (args.timesteps or 8000) * 0.025
    if args.impl == "reference":
        if rank != 0:
            return
        vals = []
        for _ in range(args.steps):
            net, n = random_network(64, seed=3, dtype=torch.float32, device="cpu",
                                    t_stop_ms=t_stop)
            pd = net.problem_dict(n)
            t0 = time.perf_counter()
            oracle.net_run(pd, n)
            dt = time.perf_counter() - t0
            vals.append(net.N * n / dt)
        v = float(np.median(vals))
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": "c3-branched-network", "sample_cells": 64},
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": 1, "kind": "port",
                             "sample": f"64-cell network, {n} steps"},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    from dendra_gb300.autotune import tune_network

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    net, n = random_network(n_cells, seed=2024 + rank, dtype=torch.float32, device=dev,
                            t_stop_ms=t_stop)
    comp_steps = net.N * n
    st = torch.cuda.current_stream(dev)
    flush = torch.ones(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    wpb, tune_ms = tune_network(net)
    # the whole run's window loop, captured once as a CUDA graph
    net.reset()
    cap = net.capture(n)
    for _ in range(max(3, args.warmup)):
        net.reset()
        cap.replay()
    torch.cuda.synchronize()
    times, spikes = [], 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            net.reset()
            flush.sum()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            r = cap.replay()
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            spikes = int(r.sum())
    ms = float(np.mean(times))
    # the same run launched window by window from the host, for comparison
    net.reset()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    net.run(n)
    e1.record(st)
    e1.synchronize()
    eager_ms = e0.elapsed_time(e1)
    value = comp_steps * world / (ms * 1e-3)
    peak, peak_kind = _peaks()
    achieved = C3_BYTES_PER_COMP_STEP * comp_steps / (ms * 1e-3) / 1e9
    windows = -(-n // net.window)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "c3-branched-network", "n_cells": n_cells,
                   "compartments": net.N, "synapses": net.n_syn, "timesteps": n,
                   "window_steps": net.window, "l2": "flushed between timed steps",
                   "launch": f"one CUDA graph of {cap.launches} kernels per run",
                   "threads_per_cell": wpb[0], "warps_per_block": wpb[1],
                   "autotune_ms": None if tune_ms is None else
                   {f"{k[0]}x{k[1]}": v for k, v in tune_ms.items()}},
        "eager_launch_ms_per_step": eager_ms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "note": f"{C3_BYTES_PER_COMP_STEP} algorithmic B per compartment-step of the "
                             f"unfused tree step; peak {peak_kind}"},
        "gpu_launches": args.steps * cap.launches, "spikes_per_run": spikes,
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu:
        cnet, cn = random_network(64, seed=3, dtype=torch.float32, device="cpu",
                                  t_stop_ms=min(t_stop, 50.0))
        pd = cnet.problem_dict(cn)
        t0 = time.perf_counter()
        oracle.net_run(pd, cn)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": cnet.N * cn / dt, "unit": METRIC, "cores": 1,
                                "kind": "port",
                                "sample": f"64-cell network ({cnet.N} compartments), {cn} steps, "
                                          "float32, one core (the network oracle is serial)"}
    if rank == 0:
        print(json.dumps(line), flush=True)


# adjoint launch, per compartment-step: tape read (v, m, h, n) 16 B + adjoint
# state read and write 32 B (the unfused reverse step's traffic)
C4_ADJ_BYTES_PER_COMP_STEP = 48


def _c4_cpu(n_sample, n_steps, seed=4):
    """Oracle forward + reverse sweep of the 1,024-cable gradient fit on a sample of
    cables.

    Returns (seconds, compartment-steps, threads)."""
    import torch

    import oracle
    from dendra_gb300.workloads import cable_population_c4

    pop, spec = cable_population_c4(n_sample, seed=seed, dtype=torch.float32, device="cpu")
    p = pop.problem_dict()
    p["rec_idx"] = np.zeros(pop.B, dtype=np.int32)
    rng = np.random.default_rng(0)
    tg = rng.standard_normal((pop.B, n_steps + 1)).astype(np.float32) * 1e-3
    t0 = time.perf_counter()
    oracle.cable_grad(p, n_steps, tg)
    return time.perf_counter() - t0, pop.N * n_steps, oracle.num_threads()


def bench_c4(args, world, rank, local):
    """1,024-cable gradient fit: seconds per gradient iteration (forward with checkpoints every
    500 steps + checkpointed recompute + adjoint) of an MSE fit of somatic
    traces, 1,024 HH cables x 201 compartments, float32, dt 0.025 ms,
    20,000 steps; gradients w.r.t. per-cable gnabar, gkbar, gl and Ra."""
    import torch

    from dendra_gb300.adjoint import CableGradient, cable_traces
    from dendra_gb300.workloads import C4_CHECKPOINT, C4_STEPS, cable_population_c4

    n_cables = min(args.cables, 1024) if args.cables != 16384 else 1024
    n_ts = args.timesteps or C4_STEPS
    full_units = n_cables * 201 * n_ts
    sample, sample_steps = 64, 2000
    cfg = {"workload": "c4-adjoint-hh-fit", "n_cables": n_cables * world, "K": 201,
           "dt_ms": 0.025, "timesteps": n_ts, "checkpoint_every": C4_CHECKPOINT,
           "params": "per-cable gnabar, gkbar, gl, Ra", "loss": "MSE of somatic traces"}
    if args.impl == "reference":
        if rank != 0:
            return
        secs = []
        for _ in range(args.steps):
            dt, units, cores = _c4_cpu(sample, sample_steps)
            secs.append(dt * full_units / units)
        v = float(np.median(secs))
        print(json.dumps({
            "impl": "reference", "metric": "grad s/iter", "value": v, "unit": "s/iter",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": "s/iter", "cores": cores, "kind": "port",
                             "sample": f"{sample} cables x {sample_steps} steps forward + reverse, "
                                       "scaled to the full workload by compartment-steps"},
            "e2e": {"value": v, "unit": "s/iter", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pop, spec = cable_population_c4(n_cables, seed=4 + rank, device=dev,
                                    fast_math=not args.exact)
    _apply_launch(pop, args.launch)
    run = CableGradient(pop, n_ts, rec_idx=0, checkpoint_every=C4_CHECKPOINT)
    names = ("gnabar", "gkbar", "gl", "ra")
    hidden = [torch.as_tensor(spec["hidden"][k], dtype=torch.float32, device=dev) for k in names]
    guess = [torch.as_tensor(spec["guess"][k], dtype=torch.float32, device=dev) for k in names]
    run.set_params(*hidden)
    target = run.forward().clone()
    n_seg = -(-n_ts // C4_CHECKPOINT)

    def grad_step(params, tgt):
        prm = [t.detach().requires_grad_() for t in params]
        trace = cable_traces(run, *prm)
        loss = ((trace - tgt) ** 2).mean()
        loss.backward()
        return loss, [t.grad for t in prm]

    for _ in range(max(3, args.warmup)):
        grad_step(guess, target)
    torch.cuda.synchronize()
    flush = torch.ones(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    times = []
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.sum()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            loss, grads = grad_step(guess, target)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    # the dominant kernel alone: one segment's adjoint launch, timed with events
    seg_k = n_seg - 1
    step0, steps = run._segments()[seg_k]
    work = tuple(c.clone() for c in run.checkpoints[seg_k])
    import ctypes

    from dendra_gb300 import _lib
    L = _lib.load()
    args_f = run._args(steps, step0, work)
    _lib.check(L.dgb_cable_run_taped(args_f, run._tapes[0].data_ptr(), _lib.stream_ptr(dev)),
               "dgb_cable_run_taped")
    adj = _lib.CableAdjointArgs()
    bufs = [torch.zeros(pop.N, device=dev) for _ in range(8)]
    gt = torch.zeros((pop.B, n_ts + 1), device=dev)
    adj.tape, adj.trace_grad, adj.trace_len = run._tapes[0].data_ptr(), gt.data_ptr(), n_ts + 1
    (adj.lam_v, adj.lam_m, adj.lam_h, adj.lam_n, adj.grad_gnabar, adj.grad_gkbar, adj.grad_gl,
     adj.grad_axial) = (b.data_ptr() for b in bufs)
    adj_ms = []
    for i in range(6):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        _lib.check(L.dgb_cable_adjoint(args_f, ctypes.byref(adj), _lib.stream_ptr(dev)),
                   "dgb_cable_adjoint")
        e1.record(st)
        e1.synchronize()
        if i >= 2:
            adj_ms.append(e0.elapsed_time(e1))
    adj_ms = float(np.mean(adj_ms))
    peak, peak_kind = _peaks()
    achieved = C4_ADJ_BYTES_PER_COMP_STEP * pop.N * steps / (adj_ms * 1e-3) / 1e9

    # ---- end to end: parameters and targets from pinned host memory, loss and
    # gradients back to the host, every iteration
    h_params = [t.cpu().pin_memory() for t in guess]
    h_target = target.cpu().pin_memory()
    d_params = [torch.empty_like(t) for t in guess]
    d_target = torch.empty_like(target)
    h_out = torch.empty(1 + 4 * pop.B, dtype=torch.float32).pin_memory()
    h2d = sum(t.numel() * 4 for t in h_params) + h_target.numel() * 4
    d2h = h_out.numel() * 4

    def e2e_step():
        for d, h in zip(d_params, h_params):
            d.copy_(h, non_blocking=True)
        d_target.copy_(h_target, non_blocking=True)
        loss, grads = grad_step(d_params, d_target)
        out = torch.cat([loss.reshape(1)] + [g.float() for g in grads])
        h_out.copy_(out, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    line = {
        "metric": "grad s/iter", "value": ms * 1e-3, "unit": "s/iter", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {**cfg, "l2": "flushed between timed steps",
                   "math": "exact" if args.exact else
                   "fast (float32 gradient within 5e-3 of the float64 oracle, tested)"},
        "compartment_steps_per_s": 3 * full_units / (ms * 1e-3),
        "loss": float(loss), "grad_norms": [float(g.norm()) for g in grads],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "cable_adjoint_kernel", "kernel_ms": adj_ms,
                     "note": f"{C4_ADJ_BYTES_PER_COMP_STEP} algorithmic B per compartment-step "
                             f"(tape read + adjoint state r/w) x {pop.N * steps} per launch; "
                             f"on-chip bound in practice; peak {peak_kind}"},
        "e2e": {"value": e2e_s, "unit": "s/iter", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": args.steps * 3 * n_seg,
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu:
        dt, units, cores = _c4_cpu(32, 1000)
        line["cpu_baseline"] = {"value": dt * full_units / units, "unit": "s/iter",
                                "cores": cores, "kind": "port",
                                "sample": "32 cables x 1000 steps forward + reverse (oracle), "
                                          "scaled to the full workload by compartment-steps"}
    if rank == 0:
        print(json.dumps(line), flush=True)


BT_BYTES_PER_ROW = 84  # float32 block row: main 36 B + lower/upper 24 B + rhs 12 B + x 12 B
BT_NCU_TRAFFIC = 236751104 + 28013056  # dram read + write of one 16,384 x 201 launch (ncu)


def _bt_system(B, K, seed, dtype):
    import torch

    g = torch.Generator().manual_seed(seed)
    lower = -torch.rand(B, K - 1, 3, generator=g)
    upper = -torch.rand(B, K - 1, 3, generator=g)
    main = 0.3 * torch.randn(B, K, 3, 3, generator=g)
    main = main + torch.diag_embed(3.0 + torch.rand(B, K, 3, generator=g))
    rhs = torch.randn(B, K, 3, generator=g)
    return [t.to(dtype) for t in (lower, main, upper, rhs)]


def bench_bt(args, world, rank, local):
    """3x3 block-tridiagonal solves of multi-layer extracellular cables
    (intracellular v and two extracellular shells per compartment): 16,384
    systems of 201 block rows, float32.  One bench step = one batched solve.
    Inputs exceed L2 (275 MB)."""
    import torch

    import oracle
    from dendra_gb300.solvers import _block3

    B = args.cables
    K = args.timesteps or 201
    units = B * K
    metric = "compartment-solves/s"
    if args.impl == "reference":
        if rank == 0:
            arrays = [t.numpy() for t in _bt_system(B, K, 7, torch.float32)]
            _reference_solve_line(
                args, world, metric, {"workload": "bt-3x3-block-tridiagonal", "systems": B,
                                      "K": K},
                units, lambda: oracle.block3_solve(*arrays),
                f"all {B} systems x {K} block rows per step, float32 block Thomas")
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    host = _bt_system(B, K, 7 + rank, torch.float32)
    lower, main, upper, rhs = (t.to(dev) for t in host)
    for _ in range(max(3, args.warmup)):
        _block3(lower, main, upper, rhs, False)
    torch.cuda.synchronize()
    flush = torch.ones(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    times = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.sum()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            _cover_enqueue()
            e0.record(st)
            x = _block3(lower, main, upper, rhs, False)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    pinned = [t.pin_memory() for t in host]
    out = torch.empty_like(host[3]).pin_memory()
    h2d = sum(t.numel() * 4 for t in pinned)
    d2h = out.numel() * 4
    dbuf = [torch.empty_like(t, device=dev) for t in host]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for d_, h_ in zip(dbuf, pinned):
            d_.copy_(h_, non_blocking=True)
        out.copy_(_block3(*dbuf, False), non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    peak, peak_kind = _peaks()
    achieved = BT_BYTES_PER_ROW * units / (ms * 1e-3) / 1e9
    n_cpu = min(1024, B)
    t0 = time.perf_counter()
    ref = oracle.block3_solve(*(t[:n_cpu].numpy() for t in host))
    cpu_s = time.perf_counter() - t0
    err = float(np.abs(x[:n_cpu].cpu().numpy() - ref).max())
    line = {
        "metric": metric, "value": units / (ms * 1e-3), "unit": metric, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "bt-3x3-block-tridiagonal", "systems": B, "K": K,
                   "l2": "flushed between timed steps",
                   "timing": COVERED_TIMING},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "kernel": "block3_kernel",
                     "traffic": BT_NCU_TRAFFIC if (B, K) == (16384, 201) else None,
                     "note": f"{BT_BYTES_PER_ROW} algorithmic B per float32 block row (read "
                             "main, bands and rhs, write x); one warp per system, factors "
                             "in shared memory; traffic = DRAM read + write of one launch "
                             f"under ncu; peak {peak_kind}"},
        "e2e": {"value": units / e2e_s, "unit": metric, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": args.steps * 2,
        "clocks": clocks.summary(),
        "max_abs_diff_vs_oracle_f32": err,
        "cpu_baseline": {"value": n_cpu * K / cpu_s, "unit": metric,
                         "cores": oracle.num_threads(), "kind": "port",
                         "sample": f"{n_cpu} systems x {K} block rows, float32 block Thomas"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


TRIDIAG_BYTES_PER_ROW = 20  # float32 row: read a, b, c, d, write x
# dram read + write of one 16,384 x 401 float32 launch of tridiag_bulk_kernel (ncu)
TRIDIAG_NCU_TRAFFIC = 105026048 + 6610944


def _tridiag_system(B, K, seed, dtype):
    """B diagonally dominant cable-like systems of K rows (the shape the
    backward-Euler cable update hands its solver): off-diagonals -U[0.05, 1],
    diagonal 1 + |a| + |c| + U[0, 0.5], right-hand side N(0, 1)."""
    import torch

    g = torch.Generator().manual_seed(seed)
    a = -(0.05 + 0.95 * torch.rand(B, K - 1, generator=g, dtype=torch.float64))
    c = -(0.05 + 0.95 * torch.rand(B, K - 1, generator=g, dtype=torch.float64))
    b = 1.0 + 0.5 * torch.rand(B, K, generator=g, dtype=torch.float64)
    b[:, 1:] -= a
    b[:, :-1] -= c
    d = torch.randn(B, K, generator=g, dtype=torch.float64)
    return [t.to(dtype).contiguous() for t in (a, b, c, d)]


def bench_tridiag(args, world, rank, local):
    """The drop-in batched tridiagonal solve (thomas_solve_cuda_t's kernel,
    dgb_tridiag_solve): 16,384 systems of 401 rows (the largest cable of the
    uneven population), float32.  One bench step = one batched solve; L2 is
    flushed between steps."""
    import torch

    import oracle
    from dendra_gb300 import _lib
    from dendra_gb300.solvers import _solve, thomas_solve_cuda_t

    B = args.cables
    K = args.timesteps or 401
    units = B * K
    metric = "row-solves/s"
    if args.impl == "reference":
        if rank == 0:
            arrays = [t.numpy() for t in _tridiag_system(B, K, 11, torch.float32)]
            _reference_solve_line(
                args, world, metric, {"workload": "tridiag-cable-systems", "systems": B, "K": K},
                units, lambda: oracle.thomas(*arrays),
                f"all {B} systems x {K} rows per step, float32 sequential Thomas")
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    host = _tridiag_system(B, K, 11 + rank, torch.float32)
    a, b, c, d = (t.to(dev) for t in host)
    for _ in range(max(3, args.warmup)):
        _solve(a, b, c, d, _lib.THOMAS)
    torch.cuda.synchronize()
    flush = torch.ones(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    times = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.sum()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            _cover_enqueue()
            e0.record(st)
            x = _solve(a, b, c, d, _lib.THOMAS)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    # end to end through the drop-in callable, from and to pinned host memory
    pinned = [t.pin_memory() for t in host]
    out = torch.empty_like(host[3]).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in pinned)
    d2h = out.numel() * out.element_size()
    dbuf = [torch.empty_like(t, device=dev) for t in host]

    def e2e_step():
        for d_, h_ in zip(dbuf, pinned):
            d_.copy_(h_, non_blocking=True)
        out.copy_(thomas_solve_cuda_t(*dbuf), non_blocking=True)

    for _ in range(max(3, args.warmup)):  # the public op's first dispatches
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    peak, peak_kind = _peaks()
    achieved = TRIDIAG_BYTES_PER_ROW * units / (ms * 1e-3) / 1e9
    n_cpu = B
    sample = [t[:n_cpu].numpy() for t in host]
    t0 = time.perf_counter()
    ref = oracle.thomas(*sample)
    cpu_s = time.perf_counter() - t0
    err = float(np.abs(x[:n_cpu].cpu().numpy() - ref).max())
    line = {
        "metric": metric, "value": units / (ms * 1e-3), "unit": metric, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "tridiag-cable-systems", "systems": B, "K": K,
                   "l2": "flushed between timed steps (256 MiB read, outside the events)",
                   "timing": COVERED_TIMING},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "kernel": "tridiag_bulk_kernel",
                     "traffic": TRIDIAG_NCU_TRAFFIC if (B, K) == (16384, 401) else None,
                     "note": f"{TRIDIAG_BYTES_PER_ROW} algorithmic B per float32 row (read "
                             "a, b, c, d, write x); traffic = DRAM read + write of one "
                             f"launch under ncu; peak {peak_kind}"},
        "e2e": {"value": units / e2e_s, "unit": metric, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": args.steps * 2,
        "clocks": clocks.summary(),
        "max_abs_diff_vs_oracle_f32": err,
        "cpu_baseline": {"value": n_cpu * K / cpu_s, "unit": metric,
                         "cores": oracle.num_threads(), "kind": "port",
                         "sample": f"{n_cpu} systems x {K} rows, float32 Thomas"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


TREE_BYTES_PER_NODE = 16  # float32: read d, g, rhs, write x
TREE_NCU_TRAFFIC = 196502528 + 12083200  # dram read + write of one 8,192-row launch (ncu)


def _tree_systems(B, seed, K=2000):
    """B Hines systems on one random branched cell of ~K compartments (branch
    lengths U[20,200] um, <= 12 branch levels): shunt cm/dt*area + g_pas*area,
    axial conductances from Ra = 100 ohm cm, right-hand sides of a voltage
    field; float32, (B, K) node order with the soma first."""
    from dendra_gb300.network import axial_conductance, random_cell

    rng = np.random.default_rng(seed)
    cell = random_cell(rng, K)
    K = cell.parent.size
    area = np.pi * cell.diam * cell.length * 1e-8                   # cm^2
    shunt = (1e-6 * 1.0 / (0.025 * 1e-3) + 1e-3) * area             # S
    axial = axial_conductance(cell.parent, cell.length, cell.diam, 100.0)
    axial[0] = 0.0
    d = shunt[None, :] * rng.uniform(0.9, 1.1, (B, K))
    g = np.broadcast_to(axial, (B, K)).copy()
    v = rng.uniform(-70.0, -50.0, (B, K))
    rhs = d * v
    return cell.parent, [np.ascontiguousarray(a, dtype=np.float32) for a in (d, g, rhs)]


def bench_tree(args, world, rank, local):
    """Tree solves of branched cells: B = 8192 systems sharing one ~2000-node
    topology (the C3 cell morphology), float32; one bench step = one batched
    tree-contraction solve (segments of <= 16 interior nodes, rake/compress
    rounds).  The DHS solve of the same systems (dhs_solve_cuda, chain
    schedule) is timed beside it.  Inputs exceed L2 (262 MB)."""
    import torch

    import oracle
    from dendra_gb300.contraction import TreeContractionPlan, solve
    from dendra_gb300.tree import build_dhs_layers, build_morphology, dhs_solve_cuda

    B = args.cables if args.cables != 16384 else 8192
    metric = "node-solves/s"
    if args.impl == "reference":
        if rank == 0:
            parent, host = _tree_systems(B, 13)
            K = parent.size
            _, _, depth = build_morphology([int(p) for p in parent])
            order, layer_ptr = build_dhs_layers(depth, 32)
            order, layer_ptr = order.numpy(), layer_ptr.numpy()
            _reference_solve_line(
                args, world, metric, {"workload": "tree-contraction-solve", "systems": B, "K": K},
                B * K, lambda: oracle.dhs_solve(*host, parent, order, layer_ptr),
                f"all {B} systems x {K} nodes per step, float32 sequential DHS (C restatement; "
                "the reference's CPU tree solvers live in the absent dendra-solvers package)")
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    parent, host = _tree_systems(B, 13 + rank)
    K = parent.size
    units = B * K
    plan = TreeContractionPlan(parent, 16)
    d, g, rhs = (torch.as_tensor(t).to(dev) for t in host)
    _, _, depth = build_morphology([int(p) for p in parent])
    order, layer_ptr = build_dhs_layers(depth, 32)
    topo = (torch.as_tensor(parent).to(dev), order.to(dev), layer_ptr.to(dev))
    for _ in range(max(3, args.warmup)):
        solve(d, g, rhs, plan)
        dhs_solve_cuda(d, g, rhs, *topo)
    torch.cuda.synchronize()
    flush = torch.ones(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)

    def timed(fn):
        out, times = None, []
        for _ in range(args.steps):
            flush.sum()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            _cover_enqueue()
            e0.record(st)
            out = fn()
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        return out, float(np.mean(times))

    with ClockSampler(local) as clocks:
        x, ms = timed(lambda: solve(d, g, rhs, plan))
        x_dhs, ms_dhs = timed(lambda: dhs_solve_cuda(d, g, rhs, *topo))
    pinned = [torch.as_tensor(t).pin_memory() for t in host]
    out = torch.empty(B, K, dtype=torch.float32).pin_memory()
    h2d = sum(t.numel() * 4 for t in pinned)
    d2h = out.numel() * 4
    dbuf = [torch.empty_like(t, device=dev) for t in pinned]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for d_, h_ in zip(dbuf, pinned):
            d_.copy_(h_, non_blocking=True)
        out.copy_(solve(*dbuf, plan), non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    peak, peak_kind = _peaks()
    achieved = TREE_BYTES_PER_NODE * units / (ms * 1e-3) / 1e9
    n_cpu = min(1024, B)
    t0 = time.perf_counter()
    ref = oracle.dhs_solve(*(t[:n_cpu] for t in host), parent, order.numpy(), layer_ptr.numpy())
    cpu_s = time.perf_counter() - t0
    xs = x[:n_cpu].cpu().numpy()
    rel = float(np.abs(xs - ref).max() / np.abs(ref).max())
    exact = oracle.tree_contract_solve(*(t[:4] for t in host), plan.tables)
    c = plan.counts
    line = {
        "metric": metric, "value": units / (ms * 1e-3), "unit": metric, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "tree-contraction-solve", "systems": B, "K": K,
                   "segment_cap": 16, "segments": c["n_segments"], "retained": c["n_retained"],
                   "rounds": c["n_rounds"], "l2": "flushed between timed steps",
                   "timing": COVERED_TIMING},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": TREE_NCU_TRAFFIC if B == 8192 else None,
                     "kernel": "tree_contract_kernel",
                     "note": f"{TREE_BYTES_PER_NODE} algorithmic B per float32 node (read d, "
                             "g, rhs, write x); one block per system, the row and its "
                             "scratch in shared memory; traffic = DRAM read + write of one "
                             f"8,192-row launch under ncu; peak {peak_kind}"},
        "e2e": {"value": units / e2e_s, "unit": metric, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": args.steps,
        "clocks": clocks.summary(),
        "dhs_same_systems": {"ms_per_step": ms_dhs, "value": units / (ms_dhs * 1e-3),
                             "kernel": "dhs_forest_kernel (chain schedule, one warp per tree)"},
        "max_rel_diff_vs_cpu_dhs_f32": rel,
        "bit_exact_vs_oracle_rows_0_3": bool(np.array_equal(x[:4].cpu().numpy(), exact)),
        "agrees_with_gpu_dhs_rel": float((x - x_dhs).abs().max() / x_dhs.abs().max()),
        "cpu_baseline": {"value": n_cpu * K / cpu_s, "unit": metric,
                         "cores": oracle.num_threads(), "kind": "port",
                         "sample": f"{n_cpu} systems x {K} nodes, float32 sequential DHS "
                                   "(C restatement; the reference's CPU tree solvers live in "
                                   "the absent dendra-solvers package)"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def _delay_bytes(n_edges, width, n_src, depth, steps, elem=4):
    """Algorithmic bytes of the direct rollout's forward launch and of its
    reverse launch (sweep + per-source sum), one edge per column, an empty
    starting ring."""
    edge_ops = n_edges * (4 + 4 + 4 + 4 + 8 + 8 + 8)  # w, f, two tap rows, source, plan
    fwd = steps * width * elem + depth * width * elem + steps * n_src * elem + edge_ops
    rev = (steps * width * elem            # delivered-row cotangents in
           + 2 * steps * n_edges * elem    # per-edge gate cotangents out and back in
           + 2 * steps * n_src * elem      # gates in, gate cotangents out
           + depth * width * elem          # ring cotangent out
           + edge_ops + 2 * n_edges * elem + n_edges * 8)  # dw, df, source plan
    return fwd, rev


def _delay_case(n_conn, n_src, depth, seed, dt_ms=0.025):
    """The 4,096-cell network's connectivity as a transport rollout: n_conn connections from
    n_src sources, each into its own synapse slot (width n_conn, post slots
    shuffled), delays U[1,5] ms at dt 0.025 ms (positions 40-200 steps),
    lognormal(-7, 0.5) weights."""
    rng = np.random.default_rng(seed)
    post = rng.permutation(n_conn)
    pre = rng.integers(0, n_src, n_conn)
    pos = np.maximum(rng.uniform(1.0, 5.0, n_conn) / dt_ms, 1.0).astype(np.float32)
    off = np.floor(pos).astype(np.int64)
    frac = (pos - off).astype(np.float32)
    w = rng.lognormal(-7.0, 0.5, n_conn).astype(np.float32)
    lower = (off % depth) * n_conn + post
    upper = (lower + n_conn) % (depth * n_conn)
    return post, pre, frac, w, lower, upper


def _delay_gates(steps, n_src, seed, rate_hz=5.0, dt_ms=0.025):
    """Per-step source gates: 0/1 spikes of independent 5 Hz sources."""
    rng = np.random.default_rng(seed)
    return (rng.random((steps, n_src)) < rate_hz * dt_ms * 1e-3).astype(np.float32)


def bench_delay(args, world, rank, local):
    """Differentiable event transport (interpolated two-tap delays) at the 4,096-cell network's
    scale: 409,600 connections from 4,096 sources into a [201][409,600] ring,
    a 2,000-step rollout forward (one launch) and its reverse sweep (one launch
    + the per-source gate reduction) through two_tap_rollout and autograd.
    The rollout starts from an empty ring.  One bench step = forward +
    backward; unit = connection-steps/s."""
    import torch

    import oracle
    from dendra_gb300 import delays

    n_conn, n_src, depth = 409_600, 4096, 201
    steps = args.timesteps or 2000
    units = n_conn * steps
    metric = "connection-steps/s"
    cfg = {"workload": "delay-two-tap-rollout", "connections": n_conn, "sources": n_src,
           "ring": [depth, n_conn], "timesteps": steps, "pass": "forward + reverse sweep",
           "l2": "flushed between timed steps"}
    if args.impl == "reference":
        if rank != 0:
            return
        post, pre, frac, w, lower, upper = _delay_case(n_conn, n_src, depth, 31)
        n_s = 100
        g = _delay_gates(n_s, n_src, 32)
        rng = np.random.default_rng(5)
        gp = rng.standard_normal((n_s, n_conn)).astype(np.float32)
        q = np.zeros((depth, n_conn), np.float32)
        vals, secs = [], 0.0
        for _ in range(args.steps):
            t0 = time.perf_counter()
            oracle.two_tap_rollout(q, 0, w, g, frac, lower, upper, pre_idx=pre)
            oracle.two_tap_rollout_vjp(q, 0, w, g, frac, lower, upper, gp, pre_idx=pre)
            secs = time.perf_counter() - t0
            vals.append(n_conn * n_s / secs)
        v = float(np.median(vals))
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": v, "unit": metric, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": units / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": v, "unit": metric, "cores": 1, "kind": "port",
                             "sample": f"all {n_conn} connections x {n_s} steps forward + "
                                       "reverse, float32, sequential ordered adds"},
            "e2e": {"value": v, "unit": metric, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    post, pre, frac, w, lower, upper = _delay_case(n_conn, n_src, depth, 31 + rank)
    gates_h = torch.from_numpy(_delay_gates(steps, n_src, 32 + rank))
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    tw, tf, tlo, tup, tpre = T(w), T(frac), T(lower), T(upper), T(pre)
    tg = gates_h.to(dev)
    gpay = torch.randn(steps, n_conn, dtype=torch.float32, device=dev,
                       generator=torch.Generator(dev).manual_seed(5))
    leaves = [t.requires_grad_() for t in (tw, tg, tf)]

    def step():
        for t in leaves:
            t.grad = None
        pay, fin = delays.two_tap_rollout(None, 0, tw, tg, tf, tlo, tup, tpre, depth=depth,
                                          width=n_conn)
        torch.autograd.backward([pay], [gpay])
        return pay

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    flush = torch.ones(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    times = []
    delays.launch_events = []  # per-launch CUDA events on the launching stream
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.sum()
            e0, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
            e0.record(st)
            step()
            e2.record(st)
            e2.synchronize()
            times.append(e0.elapsed_time(e2))
    launch_ms = {}
    for name, a, b in delays.launch_events:
        launch_ms.setdefault(name, []).append(a.elapsed_time(b))
    delays.launch_events = None
    ms = float(np.mean(times))
    ms_fwd = float(np.mean(launch_ms["two_tap_rollout"]))
    ms_rev = float(np.mean(launch_ms["two_tap_rollout_vjp"]))
    # end to end: gates in from pinned host memory, gradients out
    gates_pin = gates_h.pin_memory()
    outs = [torch.empty(n_conn, dtype=torch.float32).pin_memory() for _ in range(2)]
    gout = torch.empty(steps, n_src, dtype=torch.float32).pin_memory()
    h2d = gates_pin.numel() * 4
    d2h = (2 * n_conn + steps * n_src) * 4
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        with torch.no_grad():
            tg.copy_(gates_pin, non_blocking=True)
        step()
        outs[0].copy_(tw.grad, non_blocking=True)
        outs[1].copy_(tf.grad, non_blocking=True)
        gout.copy_(tg.grad, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    # check a prefix of the rollout against the oracle
    n_chk = 200
    pay = delays.two_tap_rollout(None, 0, tw.detach(), tg.detach()[:n_chk], tf.detach(), tlo,
                                 tup, tpre, depth=depth, width=n_conn)[0]
    t0 = time.perf_counter()
    _, opay = oracle.two_tap_rollout(np.zeros((depth, n_conn), np.float32), 0, w,
                                     gates_h[:n_chk].numpy(), frac, lower, upper, pre_idx=pre)
    cpu_s = time.perf_counter() - t0
    exact = bool(np.array_equal(pay.cpu().numpy(), opay))
    peak, peak_kind = _peaks()
    fwd_bytes, rev_bytes = _delay_bytes(n_conn, n_conn, n_src, depth, steps)
    dominant = "reverse" if ms_rev >= ms_fwd else "forward"
    kbytes, kms = (rev_bytes, ms_rev) if dominant == "reverse" else (fwd_bytes, ms_fwd)
    achieved = kbytes / (kms * 1e-3) / 1e9
    line = {
        "metric": metric, "value": units / (ms * 1e-3), "unit": metric, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": cfg,
        "forward_ms": ms_fwd, "reverse_ms": ms_rev,
        "forward_connection_steps_per_s": units / (ms_fwd * 1e-3),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "two_tap_direct_vjp_kernel + source_sum_kernel"
                     if dominant == "reverse" else "two_tap_direct_kernel",
                     "note": f"{dominant} pass, {kbytes / 1e9:.2f} GB algorithmic per launch "
                             "(reverse: delivered-row cotangents in, per-edge gate cotangents "
                             "out and back in, gates, ring cotangent, edge operands; forward: "
                             "delivered rows out, final ring, gates, edge operands), timed with "
                             f"CUDA events on its stream; peak {peak_kind}"},
        "e2e": {"value": units / e2e_s, "unit": metric, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": 4,
        "clocks": clocks.summary(),
        "bit_exact_vs_oracle": exact,
        "cpu_baseline": {"value": n_conn * n_chk / cpu_s, "unit": metric, "cores": 1,
                         "kind": "port",
                         "sample": f"forward rollout of all {n_conn} connections over "
                                   f"{n_chk} steps, float32, sequential ordered adds"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


MLP_FLOP_PER_SAMPLE = 2 * (4 * 256 + 256 * 256 + 256 * 256 + 256 * 1)


def _c5_cpu(n_fibres, seed=7, lb0=0.0, ub0=0.1, rtol=0.01):
    """Plain bisection with the Thresholder's rules (bound fixing x2 up to 10
    times, inactive lower bound, bisection to rtol, at most 25 iterations) on
    the oracle's float32 cable update, every trial simulating all open lanes.
    Returns (thresholds/s, seconds, threads)."""
    import torch

    import oracle
    from dendra_gb300.threshold import (fibre_params, fibre_population, horizon_steps,
                                        node_compartment)

    p = fibre_params(n_fibres, seed=seed)
    pop = fibre_population(p, device="cpu")
    base = pop.problem_dict()
    n_steps = horizon_steps(p["pw"].max())
    B = pop.B

    def fired(amp, lanes):
        q = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in base.items()}
        q["ve_amp"] = (-amp).astype(np.float32)
        q["spk_idx"] = np.full(B, node_compartment(5), dtype=np.int32)
        q["spk_idx2"] = np.full(B, node_compartment(-5), dtype=np.int32)
        q["spk_thr"] = 0.0
        sel = np.flatnonzero(lanes)
        if sel.size == 0:
            return np.zeros(B, dtype=bool)
        _, cnt, _, _ = oracle.cable_run(q, n_steps)
        out = np.zeros(B, dtype=bool)
        out[sel] = cnt[sel] > 0
        return out

    t0 = time.perf_counter()
    lb, ub = np.full(B, lb0), np.full(B, ub0)
    ignore = np.zeros(B, dtype=bool)
    for tries in range(11):
        act = fired(ub, ~ignore) | ignore
        if act.all():
            break
        if tries == 10:
            ignore |= ~act
            break
        ub = np.where(act, ub, ub * 2.0)
    open_ = ((ub - lb) / ub >= rtol) & ~ignore
    for _ in range(25):
        if not open_.any():
            break
        stim = (ub + lb) / 2
        f = fired(stim, open_)
        ub = np.where(open_ & f, stim, ub)
        lb = np.where(open_ & ~f, stim, lb)
        open_ = ((ub - lb) / ub >= rtol) & ~ignore
    dt = time.perf_counter() - t0
    return B / dt, dt, oracle.num_threads()


def bench_c5(args, world, rank, local):
    """65,536-fibre threshold search: thresholds/s of the learned bracket + confirming bisection vs
    plain bisection, 65,536 myelinated-fibre-like cables (241 compartments),
    rtol 1%, dt 0.005 ms, horizon = longest pulse + 4 ms.  The MLP (4 -> 256 ->
    256 -> 256 -> 1, GELU, BF16) is trained on ``--train`` plain-bisection
    thresholds first.  One bench step = one batch of thresholds."""
    import torch

    from dendra_gb300.mlp import BF16MLP, MLP_FLOPS_NOTE, fibre_features
    from dendra_gb300.threshold import (Thresholder, fibre_params, fibre_population,
                                        horizon_steps, learned_thresholds)

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    batch = min(args.cables, 65536) if args.cables != 16384 else 65536

    def plain(p):
        pop = fibre_population(p, device=dev)
        th = Thresholder(pop, lb=0.0, ub=0.1, rtol=0.01)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ub, lb = th.calculate_thresholds(horizon_steps(p["pw"].max()))
        torch.cuda.synchronize()
        return ub, lb, time.perf_counter() - t0, th

    # training data from the plain solver
    t0 = time.perf_counter()
    X, Y = [], []
    for i, s0 in enumerate(range(0, args.train, 65536)):
        n = min(65536, args.train - s0)
        p = fibre_params(n, seed=1000 + i)
        ub, _, _, _ = plain(p)
        ok = torch.isfinite(ub).cpu()
        X.append(fibre_features(p)[ok])
        Y.append(torch.log(ub.cpu()[ok]).float())
    X, Y = torch.cat(X), torch.cat(Y)
    gen_s = time.perf_counter() - t0
    mlp = BF16MLP(device=dev, seed=0)
    t0 = time.perf_counter()
    n_val = min(8192, X.shape[0] // 10)
    mlp.train(X[n_val:], Y[n_val:], epochs=30, batch=2048, lr=2e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    err = (mlp.predict(X[:n_val]).cpu().double() - Y[:n_val].double()).abs()
    margin = float(torch.quantile(err, 0.95))

    plain_t, learned_t = [], []
    agree = 0.0
    for step in range(args.warmup + args.steps):
        p = fibre_params(batch, seed=7 + step)
        pub, plb, tp, thp = plain(p)
        pop = fibre_population(p, device=dev)
        th = Thresholder(pop, lb=0.0, ub=0.1, rtol=0.01)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pred = torch.exp(mlp.predict(fibre_features(p)).double())
        lub, llb = learned_thresholds(th, pred, margin, horizon_steps(p["pw"].max()))
        torch.cuda.synchronize()
        tl = time.perf_counter() - t0
        if step >= args.warmup:
            plain_t.append(tp)
            learned_t.append(tl)
            fin = torch.isfinite(pub) & torch.isfinite(lub)
            agree = float(((llb <= pub) & (plb <= lub))[fin].float().mean())
    value = batch / float(np.mean(learned_t))
    plain_v = batch / float(np.mean(plain_t))
    # MLP inference (whole forward) and its dominant kernel, one 256x256
    # hidden layer on tcgen05, timed alone with CUDA events
    feats = fibre_features(fibre_params(batch, seed=99))
    for _ in range(3):
        mlp.predict(feats)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    xin = mlp._inputs(feats.to(dev))
    e0.record()
    for _ in range(10):
        mlp.forward(xin)
    e1.record()
    e1.synchronize()
    mlp_ms = e0.elapsed_time(e1) / 10
    from dendra_gb300.mlp import EPI_BIAS_GELU, _gemm

    h1 = torch.randn(batch, 256, device=dev).to(torch.bfloat16)
    z = torch.empty(batch, 256, device=dev)
    h2 = torch.empty(batch, 256, device=dev, dtype=torch.bfloat16)
    Wt = mlp.Wt16[1]
    layer = lambda: _gemm(batch, 256, 256, h1, 256, 1, Wt, 1, 256, bias=mlp.b[1],  # noqa: E731
                          epi=EPI_BIAS_GELU, out32=z, out16=h2)
    for _ in range(3):
        layer()
    e0.record()
    for _ in range(20):
        layer()
    e1.record()
    e1.synchronize()
    layer_ms = e0.elapsed_time(e1) / 20
    layer_tf = 2.0 * batch * 256 * 256 / (layer_ms * 1e-3) / 1e12
    peak_tf = 1927.7
    # the dominant kernel of the whole search: the fibre trial (persistent
    # cable run), one full-horizon trial of the batch without early stop
    pf = fibre_params(batch, seed=123)
    popf = fibre_population(pf, device=dev)
    ns = horizon_steps(pf["pw"].max())
    popf._dev["ve_amp"].fill_(-0.05)
    popf.run(10)
    torch.cuda.synchronize()
    e0.record()
    popf.run(ns)
    e1.record()
    e1.synchronize()
    trial_ms = e0.elapsed_time(e1)
    trial_units = popf.N * ns
    peak, peak_kind = _peaks()
    achieved = ALG_BYTES_PER_COMP_STEP * trial_units / (trial_ms * 1e-3) / 1e9
    line = {
        "metric": "thresholds/s", "value": value, "unit": "thresholds/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(learned_t)) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "c5-learned-threshold", "batch": batch, "rtol": 0.01,
                   "training_thresholds": int(X.shape[0]), "dt_ms": 0.005,
                   "horizon": "longest pulse + 4 ms"},
        "plain_bisection": {"value": plain_v, "unit": "thresholds/s"},
        "speedup_vs_plain_bisection": value / plain_v,
        "mlp": {"median_abs_log_err": float(err.median()), "margin": margin,
                "bracket_agreement": agree, "train_s": train_s, "data_generation_s": gen_s,
                "inference_ms": mlp_ms,
                "inference_tflops": MLP_FLOP_PER_SAMPLE * batch / (mlp_ms * 1e-3) / 1e12,
                "roofline": {"bound": "tensor", "kernel": "gemm_tc_kernel (one 256x256 layer)",
                             "achieved": layer_tf, "peak": peak_tf, "unit": "TFLOP/s",
                             "frac": layer_tf / peak_tf, "kernel_ms": layer_ms,
                             "note": MLP_FLOPS_NOTE + "; peak: measured cuBLAS bf16 burst"}},
        "roofline": {"bound": "hbm", "kernel": "cable_run_kernel (fibre trials)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "kernel_ms": trial_ms,
                     "note": f"{ALG_BYTES_PER_COMP_STEP} algorithmic B per compartment-step "
                             f"x {trial_units} compartment-steps of one full-horizon trial of "
                             f"the batch; peak {peak_kind} copy bandwidth"},
    }
    if rank == 0 and not args.no_cpu:
        v, secs, cores = _c5_cpu(64)
        line["cpu_baseline"] = {"value": v, "unit": "thresholds/s", "cores": cores,
                                "kind": "port",
                                "sample": "64 fibres, plain bisection on the oracle's float32 "
                                          "cable update (all open lanes simulated per trial)"}
    if rank == 0:
        print(json.dumps(line), flush=True)


# the other configurations, measured by the default run after the 16,384-cable population (one
# child process each, their own JSON lines summarised): workload, extra
# arguments, time limit in seconds
OTHER_CONFIGS = (("c1", ["--steps", "3"], 300), ("c3", [], 600), ("c4", ["--steps", "2"], 600),
                 ("c5", [], 900), ("tridiag", ["--steps", "20"], 300))
OTHER_KEYS = ("metric", "value", "unit", "ms_per_step", "higher_is_better", "dtype", "config",
              "e2e", "clocks", "gpu_launches", "accuracy", "fp32_vs_fp64")


def _other_configs():
    """Run every other configuration's bench in a child process (3 warm-up
    steps, then one timed step, or more where a step is short; no CPU
    baseline) and keep each line's
    measurement, roofline and accuracy keys; a child that fails is recorded
    with its error."""
    out = {}
    for wl, extra, limit in OTHER_CONFIGS:
        cmd = [sys.executable, os.path.abspath(__file__), "--workload", wl, "--steps", "1",
               "--warmup", "3", "--no-cpu", "--no-configs", *extra]
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=limit,
                               env=dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0"))
            lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            if r.returncode != 0 or not lines:
                tail = (r.stderr or r.stdout).strip().splitlines()[-1:] or [""]
                out[wl] = {"error": f"exit {r.returncode}: {tail[0][:300]}"}
                continue
            d = json.loads(lines[-1])
            rec = {k: d[k] for k in OTHER_KEYS if k in d}
            if "roofline" in d:
                rec["roofline"] = {k: d["roofline"].get(k) for k in
                                   ("bound", "achieved", "peak", "unit", "frac", "kernel")}
            for k in d:
                if k.startswith("speedup") or k in ("threshold_rtol", "spikes_per_run"):
                    rec[k] = d[k]
            rec["wall_s"] = time.perf_counter() - t0
            out[wl] = rec
        except subprocess.TimeoutExpired:
            out[wl] = {"error": f"no result within {limit} s"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--sample", type=int, default=512, help="CPU baseline cables")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the child runs of the other workloads after the default one")
    ap.add_argument("--exact", action="store_true",
                    help="exact float32 arithmetic instead of the fast-math variant")
    ap.add_argument("--workload", default="c2",
                    choices=["c1", "c2", "c3", "c4", "c5", "bt", "delay", "tree", "tridiag"],
                    help="c1: 64 x 101 float64 cables with full traces and rasters; "
                         "c2: uneven cable population (default); c3: branched-cell network; "
                         "c4: adjoint gradient of a trace fit; "
                         "c5: learned threshold proposal vs plain bisection; "
                         "bt: 3x3 block-tridiagonal (multi-layer extracellular) solves; "
                         "delay: differentiable two-tap event transport rollout; "
                         "tree: tree-contraction solves of branched cells; "
                         "tridiag: the drop-in batched tridiagonal solve")
    ap.add_argument("--train", type=int, default=200000, help="c5 training thresholds")
    ap.add_argument("--cables", type=int, default=16384,
                    help="cables per rank (a smaller case for profiling)")
    ap.add_argument("--timesteps", type=int, default=0, help="timesteps per run (default 2000)")
    ap.add_argument("--ref-steps", type=int, default=100,
                    help="timesteps of each reference CPU sample (reference arm)")
    ap.add_argument("--ref-child", default="", help=argparse.SUPPRESS)
    ap.add_argument("--launch", default="",
                    help="c2: fixed 'wpb,k16,k8' instead of autotuning (profiling runs); "
                         "c1, c4: the first field fixes the cables per CTA (-1: split gates)")
    args = ap.parse_args()
    if args.ref_child:
        return _ref_child(args.ref_child, args.ref_steps, args.steps, args.warmup)
    world, rank, local = _dist()
    if args.workload == "c1":
        return bench_c1(args, world, rank, local)
    if args.workload == "c3":
        return bench_c3(args, world, rank, local)
    if args.workload == "c4":
        return bench_c4(args, world, rank, local)
    if args.workload == "bt":
        return bench_bt(args, world, rank, local)
    if args.workload == "c5":
        return bench_c5(args, world, rank, local)
    if args.workload == "delay":
        return bench_delay(args, world, rank, local)
    if args.workload == "tree":
        return bench_tree(args, world, rank, local)
    if args.workload == "tridiag":
        return bench_tridiag(args, world, rank, local)
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch

    import dendra_gb300
    from dendra_gb300.shards import reduce_timing
    from dendra_gb300.workloads import C2_STEPS, cable_population_c2

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    dendra_gb300.load()

    # each rank owns an independent shard of cables (weak scaling, no collective)
    n_ts = args.timesteps or C2_STEPS
    pop = cable_population_c2(n_cables=args.cables, dtype=torch.float32, device=dev,
                              seed=2024 + rank, fast_math=not args.exact)
    comp_steps = pop.N * n_ts
    from dendra_gb300.autotune import tune_cable_run

    if args.launch:
        wpb, tune_ms = tuple(int(x) for x in args.launch.split(",")), None
        _apply_launch(pop, args.launch)
        pop.lanes_split = None if wpb[1:] == (0, 0) else wpb[1:]
    else:
        wpb, tune_ms = tune_cable_run(pop, n_steps=100)
    v0, m0, h0, n0 = (t.clone() for t in (pop.v, pop.m, pop.h, pop.n))

    def reset():
        pop.v.copy_(v0)
        pop.m.copy_(m0)
        pop.h.copy_(h0)
        pop.n.copy_(n0)
        pop.step_index = 0

    flush = torch.ones(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)

    def one(spk=False):
        reset()
        return pop.run(n_ts, spk_idx=0 if spk else None)

    for _ in range(max(3, args.warmup)):
        one()
    torch.cuda.synchronize()
    pop.check_status()

    def barrier():
        if pg is not None:
            pg.barrier()

    times = []
    with ClockSampler(local) as clocks:
        barrier()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            reset()
            flush.sum()  # evict L2 between timed steps (outside the events; read: no dirty lines)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            pop.run(n_ts, spk_idx=0)  # with the spike detection (count and first step)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        barrier()
    ms = float(np.mean(times))
    # slowest rank's time, work summed over ranks (unchanged at one rank)
    ms, total_units = reduce_timing(ms, comp_steps, device=dev)
    value = total_units / (ms * 1e-3)

    # ---- end-to-end through the public API from pinned host buffers ----
    host_in = {k: v.detach().cpu().pin_memory() for k, v in pop._dev.items()}
    host_state = {k: t.cpu().pin_memory() for k, t in (("v", v0), ("m", m0), ("h", h0), ("n", n0))}
    h2d = sum(t.numel() * t.element_size() for t in host_in.values())
    h2d += sum(t.numel() * t.element_size() for t in host_state.values())
    out_v = torch.empty(pop.N, dtype=pop.dtype).pin_memory()
    out_cnt = torch.empty(pop.B, dtype=torch.int32).pin_memory()
    out_first = torch.empty(pop.B, dtype=torch.int32).pin_memory()
    d2h = sum(t.numel() * t.element_size() for t in (out_v, out_cnt, out_first))

    def e2e_step():
        for k, t in host_in.items():
            pop._dev[k].copy_(t, non_blocking=True)
        for k, t in host_state.items():
            getattr(pop, k).copy_(t, non_blocking=True)
        pop.step_index = 0
        res = pop.run(n_ts, spk_idx=0)
        out_v.copy_(pop.v, non_blocking=True)
        out_cnt.copy_(res.spk_count, non_blocking=True)
        out_first.copy_(res.spk_first, non_blocking=True)

    e2e_ms = float("nan")
    if not args.no_e2e:
        e2e_step()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_ms, _ = reduce_timing(e2e_ms, 0, device=dev)
    e2e_value = total_units / (e2e_ms * 1e-3)
    n_spiking = int((out_cnt > 0).sum())

    # ---- the plain per-step path (assemble + solve/update per timestep) ----
    plain = None
    if not args.no_plain:
        reset()
        bands = torch.empty((4, pop.N), dtype=pop.dtype, device=dev)
        for _ in range(3):
            pop.step_plain(bands)
        reset()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        n_plain = 200
        e0.record(st)
        for _ in range(n_plain):
            pop.step_plain(bands)
        e1.record(st)
        e1.synchronize()
        pms = e0.elapsed_time(e1) / n_plain
        plain = {"value": pop.N / (pms * 1e-3), "unit": METRIC, "ms_per_timestep": pms,
                 "timesteps_timed": n_plain,
                 "what": "dgb_cable_assemble + dgb_cable_solve_update per timestep (2 launches)"}

    # ---- the reference's eager per-step structure (one kernel per op) ----
    eager = None
    if not args.no_plain:
        reset()
        bands = torch.empty((4, pop.N), dtype=pop.dtype, device=dev)
        for i in range(3):
            eager_reference_step(pop, bands, i)
        reset()
        torch.cuda.synchronize()
        n_eager = 50
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for i in range(n_eager):
            eager_reference_step(pop, bands, i)
        e1.record(st)
        e1.synchronize()
        ems = e0.elapsed_time(e1) / n_eager
        # same first 20 timesteps through the eager structure and the 2-kernel path
        reset()
        for i in range(20):
            eager_reference_step(pop, bands, i)
        v_eager = pop.v.clone()
        reset()
        for i in range(20):
            pop.step_plain(bands)
        dv = float((pop.v - v_eager).abs().max())
        eager = {"value": pop.N / (ems * 1e-3), "unit": METRIC, "ms_per_timestep": ems,
                 "timesteps_timed": n_eager, "max_abs_dv_vs_plain_mv_20_steps": dv,
                 "what": "the reference's eager step structure: one torch kernel per "
                         "elementwise op of the gate advance, current frame and assembly, "
                         "then the ragged solve + update kernel"}
        reset()

    # ---- the reference's own GPU path on the same GPU (Triton Thomas solve +
    #      eager mechanism kernels per step), on the population's equal-K groups ----
    ref_gpu = None
    if rank == 0 and not args.no_plain:
        r = reference_cpu("c2gpu", 200, reps=3, warmup=1)
        if "error" in r:
            ref_gpu = {"unavailable": r["error"]}
        else:
            secs = float(np.median(r["times"]))
            ref_gpu = {"value": r["units"] / secs, "unit": METRIC, "seconds": secs,
                       "what": (f"the reference's model.run on this GPU at JIT=0 (Triton "
                                "thomas_solve_cuda_t + eager mechanism kernels per step), "
                                f"16,384-cable population groups K={list(C2_REF_GROUPS)} "
                                f"({sum(g[1] for g in r['groups'])} cables, one Unmyelinated "
                                "population per K) x 200 timesteps, float32")}

    peak, peak_kind = _peaks()
    achieved = ALG_BYTES_PER_COMP_STEP * comp_steps / (ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "c2-uneven-hh-cables-extracellular", "n_cables": args.cables * world,
                   "compartments_per_rank": pop.N, "k_range": [51, 401], "dt_ms": 0.005,
                   "timesteps": n_ts, "state_dtype": "float32",
                   "math": "exact" if args.exact else "fast (float32 error vs float64: "
                                                       "fp32_vs_fp64)",
                   "l2": "flushed between timed steps (256 MiB read, outside the events)",
                   "launch": "one persistent dgb_cable_run launch per step",
                   "warps_per_block": wpb[0], "lanes_split_k16_k8": list(wpb[1:]),
                   "autotune_ms": None if tune_ms is None else
                   {str(k): v for k, v in tune_ms.items()}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": C2_NCU_DRAM_BYTES_PER_COMP * pop.N,
                     "note": (f"achieved = {ALG_BYTES_PER_COMP_STEP} algorithmic B per "
                              f"compartment-step of the unfused update x {comp_steps} "
                              f"compartment-steps / launch time; peak {peak_kind} copy "
                              "bandwidth; the persistent kernel keeps state on chip, so its "
                              "DRAM traffic (ncu, 4,096-cable capture, scaled by compartments: "
                              "it is read once per launch, not per step) is far below the "
                              "unfused update's")},
        "onchip": _issue_bound(C2_NCU_THREAD_INSTR_PER_COMP_STEP, comp_steps, ms, clocks, dev),
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms},
        "gpu_launches": args.steps * (1 if args.no_e2e else 2),
        "clocks": clocks.summary(),
        "cables_spiking": n_spiking,
    }
    if plain is not None:
        line["plain_gpu"] = plain
        line["speedup_vs_plain_gpu"] = value / plain["value"]
    if eager is not None:
        line["plain_eager_reference_structure"] = eager
        line["speedup_vs_plain_eager"] = value / eager["value"]
    if ref_gpu is not None:
        line["plain_reference_gpu"] = ref_gpu
        if "value" in ref_gpu:
            line["speedup_vs_plain_reference_gpu"] = value / ref_gpu["value"]
        line["gpu_launches"] += 0  # plain path runs outside the timed region
    if rank == 0 and not args.no_cpu:
        gpu_outs = _c2_gpu_outputs(dev, fast_math=not args.exact)
        v, n_comp, secs, cores = cpu_baseline(args.sample, 200)
        port = {"value": v, "unit": METRIC, "cores": cores, "kind": "port",
                "sample": f"{args.sample} of 16384 cables ({n_comp} compartments) x 200 "
                          "timesteps, float32, the oracle's C restatement"}
        cpu, why = reference_baseline("c2", 50)
        if cpu is None:
            cpu = dict(port, note=why)
        else:
            cpu.pop("seconds")
        line["cpu_baseline"] = cpu
        line["cpu_port"] = port
        line["fp32_vs_fp64"] = _c2_accuracy(gpu_outs)
    if rank == 0 and world == 1 and not args.no_configs:
        line["other_configs"] = _other_configs()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
