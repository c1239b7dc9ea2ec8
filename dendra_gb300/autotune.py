"""Project autotuner for the launch parameters of the GB300 kernels.

The reference picks its kernel configuration by hand (the DHS ``threads``
layer chunking, tree.py:169-178; the Thomas-or-PCR method choice,
implicit.py:364-440).  Here each knob is a parameter of the C ABI and is
chosen by timing the candidates on the device:

* cables per CTA of the persistent cable kernels (``dgb_cable_args.
  warps_per_block``: 1, 2 or 4), the split-gate run (``DGB_CABLE_SPLIT_GATES``:
  one cable on 4 warps) and the persistent run's Thomas/PCR split
  (``lanes_mode``/``n_lanes32``/``n_lanes16``: short cables on 8 or 16 lanes,
  i.e. longer sequential chunks and fewer PCR stages) — ``tune_cable_run``;
* the Thomas-versus-PCR split of the chunked tridiagonal solve (lanes per
  system 4 .. 32, i.e. rows per lane eliminated sequentially vs reduced by
  PCR) — ``tune_tridiag_lanes``;
* threads per cell and warps per CTA of the network window kernel
  (``dgb_net_args.threads_per_cell``, ``warps_per_block``: the tree-level
  tiling) — ``tune_network``.

Every candidate runs a short representative workload (warm-up, then the
median of ``reps`` timings with CUDA events on the current stream).  Results
are cached per (knob, shape key, device name) for the process; a JSON file
named by ``DGB_TUNE_CACHE`` keeps them across processes.  Launch-shape
candidates (CTA sizes, threads per cell) never change the arithmetic, so they
give identical results; the lane splits of the tridiagonal solves change the
order of the elimination and so the rounding (every split is tested against
the oracle within the solver tolerances).
"""

from __future__ import annotations

import json
import os
import threading

import torch

_lock = threading.Lock()
_cache: dict[str, object] | None = None


def _load_cache():
    global _cache
    if _cache is None:
        _cache = {}
        path = os.environ.get("DGB_TUNE_CACHE")
        if path and os.path.exists(path):
            try:
                with open(path) as f:
                    _cache.update(json.load(f))
            except (OSError, ValueError):
                pass
    return _cache


def _store(key, value):
    cache = _load_cache()
    cache[key] = value
    path = os.environ.get("DGB_TUNE_CACHE")
    if path:
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def _key(kind, device, *parts):
    name = torch.cuda.get_device_name(device).replace(" ", "_")
    return "|".join([kind, name] + [str(p) for p in parts])


def time_candidates(run, candidates, device, reps=3, warmup=1):
    """{candidate: median milliseconds} of run(candidate) timed with CUDA events."""
    st = torch.cuda.current_stream(device)
    out = {}
    for c in candidates:
        for _ in range(warmup):
            run(c)
        ts = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            run(c)
            e1.record(st)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        out[c] = sorted(ts)[len(ts) // 2]
    return out


def tune(kind, key_parts, candidates, run, device, reps=3, force=False):
    """Best candidate for (kind, key) — cached — and the timings if measured now."""
    key = _key(kind, device, *key_parts)
    with _lock:
        cache = _load_cache()
        if not force and key in cache:
            v = cache[key]
            return (tuple(v) if isinstance(v, list) else v), None
    timings = time_candidates(run, candidates, device, reps=reps)
    best = min(timings, key=timings.get)
    with _lock:
        _store(key, list(best) if isinstance(best, tuple) else best)
    return best, timings


# (cables per CTA, k16, k8): cables with K <= k8 on 8 lanes, K <= k16 on 16
# lanes, the rest on 32 ((0, 0): every cable on 32 lanes).  Cables per CTA
# -1: the split-gate run (one cable per CTA of 4 warps, every cable on 32
# lanes), for populations with few cables per SM.
CABLE_RUN_SPLIT = (-1, 0, 0)
CABLE_RUN_CANDIDATES = tuple((w, k16, k8) for w in (2, 4)
                             for k16, k8 in ((0, 0), (96, 0), (128, 0), (128, 64), (160, 80))
                             ) + (CABLE_RUN_SPLIT,)


def tune_cable_run(pop, n_steps=50, candidates=CABLE_RUN_CANDIDATES, reps=3, force=False):
    """Pick cables per CTA (or the split-gate run) and the lane split for
    ``pop``'s persistent runs; sets pop.warps_per_block, pop.split_gates and
    pop.lanes_split.

    Times ``n_steps`` steps from the population's current state (restored
    after every timing).  Returns ((wpb, k16, k8), {candidate: ms} or None if
    cached)."""
    state = tuple(t.clone() for t in (pop.v, pop.m, pop.h, pop.n))
    step, t = pop.step_index, pop.t
    saved = (pop.warps_per_block, pop.split_gates, pop.lanes_split)

    def apply(c):
        w, k16, k8 = (int(x) for x in c)
        if w < 0 and (k16, k8) != (0, 0):
            raise ValueError("the split-gate run keeps every cable on 32 lanes")
        pop.warps_per_block = max(w, 0)
        pop.split_gates = w < 0
        pop.lanes_split = None if k16 == 0 and k8 == 0 else (k16, k8)

    kmax = max(pop.n_comp)
    ch = max(-(-kmax // 32), 8)
    candidates = tuple(c for c in candidates if c[1] <= 16 * ch and c[2] <= 8 * ch)

    def run(c):
        apply(c)
        for dst, src in zip((pop.v, pop.m, pop.h, pop.n), state):
            dst.copy_(src)
        pop.step_index, pop.t = step, t
        pop.run(n_steps)

    # the candidate set is part of the key: a restricted set (e.g. no lane
    # splits) never inherits a pick from a wider one
    parts = (str(pop.dtype), pop.B, kmax, pop.N, pop.fast_math, "ve" if pop.field is not None
             else "-", ";".join(f"{w}/{a}/{b}" for w, a, b in candidates))
    try:
        best, timings = tune("cable_run_split", parts, candidates, run, pop.device, reps, force)
    finally:
        for dst, src in zip((pop.v, pop.m, pop.h, pop.n), state):
            dst.copy_(src)
        pop.step_index, pop.t = step, t
        pop.warps_per_block, pop.split_gates, pop.lanes_split = saved
    best = tuple(int(x) for x in best)
    apply(best)
    return best, timings


def tune_tridiag_lanes(B, K, dtype=torch.float32, device="cuda", candidates=(4, 8, 16, 32),
                       reps=5, force=False):
    """Lanes per system for dgb_tridiag_solve_lanes on (B, K) systems.

    Few lanes = long sequential (Thomas-like) chunks per lane, many lanes =
    short chunks and a wider PCR; candidates whose rows per lane exceed the
    compiled chunk sizes are skipped."""
    from .solvers import tridiag_solve_lanes

    device = torch.device(device)
    g = torch.Generator(device="cpu").manual_seed(0)
    a = (-torch.rand(B, K - 1, generator=g, dtype=torch.float64)).to(device, dtype)
    c = (-torch.rand(B, K - 1, generator=g, dtype=torch.float64)).to(device, dtype)
    b = (3.0 + torch.rand(B, K, generator=g, dtype=torch.float64)).to(device, dtype)
    d = torch.randn(B, K, generator=g, dtype=torch.float64).to(device, dtype)
    ok = [n for n in candidates if -(-K // n) <= 33]
    return tune("tridiag_lanes", (str(dtype), B, K), ok,
                lambda n: tridiag_solve_lanes(a, b, c, d, lanes=n), device, reps, force)


def tune_network(net, n_steps=None, candidates=((32, 4), (64, 4), (128, 4), (256, 8), (512, 8)),
                 reps=2,
                 force=False):
    """Threads per cell and warps per CTA for ``net``'s window kernel (the
    tree-level tiling: how many threads share one cell's node, chain and
    synapse loops); sets net.threads_per_cell and net.warps_per_block.

    Times ``n_steps`` (default two windows) from a reset network and leaves
    the network reset.  Returns ((threads_per_cell, warps_per_block), timings)."""
    n_steps = int(n_steps or 2 * net.window)
    saved = (net.threads_per_cell, net.warps_per_block)

    def run(c):
        net.threads_per_cell, net.warps_per_block = c
        net.reset()
        net.run(n_steps)

    parts = (str(net.dtype), net.n_cells, net.N, net.plan.max_k)
    try:
        best, timings = tune("net_window_tiling", parts, candidates, run, net.device, reps,
                             force)
    finally:
        net.threads_per_cell, net.warps_per_block = saved
        net.reset()
    best = tuple(int(x) for x in best)
    net.threads_per_cell, net.warps_per_block = best
    return best, timings
