"""Benchmark of the voxel step on GB300.

Headline workload (one "step" = one 64-step segment of the batched pool):
2048 independent worlds, dims iid from {16,24,32,48,64,96,128}^3 (seeded),
stepped together by the resident segment kernels (each world takes all of a
segment's steps in one launch of its size class) inside one CUDA graph per
segment.  The same line carries:
  * value_fresh: the same worlds generated anew, one segment from step 0;
  * plain_per_world: the drop-in byte kernel launched once per world per step
    (2048 x 64 launches per segment) on the same worlds;
  * plain_512: the drop-in byte kernel on one 512^3 pillar world (HBM-bound);
  * roofline of the dominant kernel (CUDA-event time per launch), with the
    issue-rate roof beside it;
  * cpu_baseline: the CPU oracle timed on this host (bounded sample);
  * parity: results of the timed GPU runs, read back and checked against the
    oracle in the CPU leg once every GPU measurement has ended;
  * e2e / e2e_fresh: the same metric through the C ABI from pinned host
    buffers (admit = H2D + conversion, one segment, retire = conversion + D2H);
  * served, large_render, mesh_render, engine_loop: the serving loop, the
    1024^3 world with a frame per step, the mesh materials, and one step per
    call of a 64^3 world.
`--impl reference` times the CPU oracle (the upstream project has no step of
its own) on a bounded sample of the same workload with all host threads.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl fs3d|reference]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import gc
import json
import os
import re
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-updates/s: batched+served vs plain per-world launch, 1 GB300, bit-exact"
UNIT = "voxel-updates/s"
L2_FLUSH_BYTES = 512 << 20


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "samples": len(sm),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------------ workload
def batch_worlds(fs3d, master: int, count: int):
    dims, seeds = fs3d.gen_batch_dims(master, count)
    return [(tuple(int(v) for v in dims[w]), int(seeds[w])) for w in range(count)]


def pinned_views(torch, shapes):
    """One page-locked arena with a (Y, Z, X) view per world, back to back (the
    way a server keeps request payloads): the library moves such runs over the
    host link in one copy-engine transfer."""
    sizes = [int(np.prod(sh)) for sh in shapes]
    arena = torch.empty(sum(sizes), dtype=torch.uint8, pin_memory=True)
    views, off = [], 0
    for sh, n in zip(shapes, sizes):
        views.append(arena[off:off + n].view(*sh))
        off += n
    return views


def gen_grids(fs3d, worlds, pinned_torch=None):
    """Host grids (in one pinned arena when torch is given), generated in parallel."""
    def one(w):
        (X, Y, Z), seed = w
        return fs3d.gen_batch_world(seed, X, Y, Z)
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        grids = list(ex.map(one, worlds))
    if pinned_torch is not None:
        out = pinned_views(pinned_torch, [g.shape for g in grids])
        for t, g in zip(out, grids):
            t.numpy()[...] = g
        return out
    return grids


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_values(name: str, keys):
    """Named figures (`key: value` lines) from a summary under profiles/, or None."""
    try:
        txt = open(os.path.join(ROOT, "profiles", f"{name}.md")).read()
    except OSError:
        return None
    out = {}
    for k in keys:
        m = re.search(rf"{k}:\s*([0-9.eE+]+)", txt)
        if not m:
            return None
        out[k] = float(m.group(1))
    return out


def profile_traffic(kernel: str):
    """Per-launch DRAM bytes recorded from an ncu capture under profiles/."""
    path = os.path.join(ROOT, "profiles", f"{kernel}.md")
    try:
        txt = open(path).read()
    except OSError:
        return None, None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", txt)
    c = re.search(r"traffic_cells_per_launch:\s*([0-9.eE+]+)", txt)
    if not m:
        return None, None
    return float(m.group(1)), (float(c.group(1)) if c else None)


# ------------------------------------------------------------------ CPU leg: oracle timing and checks
def load_oracle():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    return oracle_lib.load()


def oracle_worlds(orc, master: int, count: int):
    """The batch's dims and seeds from the oracle's own generator."""
    dims, seeds = orc.gen_c3_dims(master, count)
    return [(tuple(int(v) for v in dims[w]), int(seeds[w])) for w in range(count)]


def oracle_sample_index(count: int):
    """The CPU legs' bounded sample: every 16th world of the batch."""
    return list(range(0, count, 16))


def run_parallel(fn, items, threads):
    """fn over items on `threads` host threads (largest items first when they
    are (grid, ...) tuples); the oracle releases the interpreter while it runs."""
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(fn, items))


def oracle_rate(orc, states, budget_s: float, threads: int, steps_each: int = 4, window: int = 64):
    """Times the oracle step on `states` ([grid, seed, step] each) for about
    budget_s: a queue of worlds, largest first; a thread takes a world, steps
    a working copy steps_each steps from where it stands and puts it back, so
    no world is held by two threads and no thread waits for a round to end.
    Every `window` steps a world starts over from its given state, so the
    timed work is the given states' next `window` steps (one segment), as the
    GPU times it.  Returns voxel-updates/s and a description."""
    import queue
    import threading
    q = queue.Queue()
    for i in sorted(range(len(states)), key=lambda i: -states[i][0].size):
        q.put(i)
    work = [[np.ascontiguousarray(g).copy(), 0] for g, _, _ in states]
    deadline = time.perf_counter() + budget_s
    done = []

    def worker():
        n = 0
        while time.perf_counter() < deadline:
            i = q.get()
            g0, seed, t0 = states[i]
            cur, k = work[i]
            if k >= window:
                np.copyto(cur, g0)
                k = 0
            Y, Z, X = cur.shape
            orc.L.orc_run(cur.ctypes.data, X, Y, Z, seed, t0 + k, steps_each, None, 1)
            work[i][1] = k + steps_each
            n += cur.size * steps_each
            q.put(i)
        done.append(n)

    t0 = time.perf_counter()
    ts = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    dt = time.perf_counter() - t0
    return sum(done) / dt, {"worlds": len(states), "steps_per_take": steps_each, "window": window,
                            "voxel_updates": int(sum(done)), "seconds": round(dt, 3)}


ORACLE_FLAGS = "gcc -O3 -fopenmp -ffp-contract=off (oracle/Makefile), one world per thread, work queue"


class OracleChecks:
    """GPU results recorded by the GPU legs (copies on the host), checked
    against the oracle in the CPU leg, after every GPU measurement has ended."""

    def __init__(self):
        self.runs = {}    # label -> [(grid before, seed, first step, steps, GPU grid after)]
        self.dda = None   # (grid, camera, W, H, GPU frame, tolerance)
        self.mesh = None  # (scene view kwargs, draws, W, H, GPU frame)

    def add_run(self, label, grid, seed, t0, n, got):
        self.runs.setdefault(label, []).append((grid, seed, t0, n, got))

    def check(self, threads):
        """Returns {"parity": str, "large": {...}, "mesh": {...}}.  Every
        recorded world is stepped by the oracle (one thread each, in
        parallel) and compared whole."""
        import oracle_lib
        orc = load_oracle()
        out, notes = {}, []

        def one(item):
            grid, seed, t0, n, got = item
            g = np.ascontiguousarray(grid).copy()
            Y, Z, X = g.shape
            orc.L.orc_run(g.ctypes.data, X, Y, Z, seed, t0, n, None, 1)
            return bool(np.array_equal(np.asarray(got), g))

        for label, items in self.runs.items():
            items = sorted(items, key=lambda it: -it[0].size)
            ok = run_parallel(one, items, threads)
            bad = len(ok) - sum(ok)
            notes.append(f"{label}: {sum(ok)} of {len(ok)} worlds bit-exact" + (f" ({bad} MISMATCH)" if bad else ""))
        out["parity"] = "; ".join(notes) if notes else None
        if self.dda is not None:
            grid, cam, W, H, got, tol = self.dda
            exp = orc.render_dda(grid, oracle_lib.camera_from(cam), W, H)
            d = float(np.abs(got - exp).max())
            out["large"] = {"last_frame_max_abs_diff_vs_cpu": d, "tolerance": tol, "within_tolerance": d <= tol}
        if self.mesh is not None:
            kw, draws, W, H, got = self.mesh
            exp = orc.render_meshes(oracle_lib.scene_view(**kw), draws, W, H)
            out["mesh"] = {"bit_exact_vs_cpu": bool(np.array_equal(got, exp))}
        return out


# untimed segments of the headline run that precede its timed ones: the
# autotuner's six (two candidate promotions, each one untimed segment and two
# timed ones; every world of the batch fits a resident class, so the per-step
# grid is not a candidate) follow the warm-up, and one plain segment follows
# them (the tuner leaves the chosen configuration freshly captured: its first
# segment rebuilds the tables and uploads the graph)
TUNE_SEGMENTS = 6


def untimed_segments(args) -> int:
    """Segments stepped before the timed ones, the same in both arms: at least
    --timed-from / --segment, more when the warm-up (at least three segments,
    so the worlds are past their young steps before tuning) and the tuner
    need them."""
    pre = max(args.warmup, 3)
    tune = 0 if args.no_autotune else TUNE_SEGMENTS
    return max(args.timed_from // args.segment, pre + tune + 1)


def run_reference(args):
    """The reference arm: the upstream project has no step of its own, so the
    CPU oracle (FS3D-rule v1) stands in, on the batch's worlds made by the
    oracle's own generators.  `value` times the states the GPU arm's timed
    segments step (every world advanced untimed to --timed-from first);
    `value_fresh` the freshly generated worlds from step 0."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    orc = load_oracle()
    threads = os.cpu_count() or 1
    start = args.segment * untimed_segments(args)  # where the GPU arm's timed segments begin
    worlds = oracle_worlds(orc, args.master, args.worlds)
    sample = [worlds[i] for i in oracle_sample_index(args.worlds)]

    def gen(w):
        (X, Y, Z), seed = w
        return [orc.gen_c3_world(seed, X, Y, Z), seed, 0]

    fresh = run_parallel(gen, sample, threads)
    settled = [[g.copy(), seed, 0] for g, seed, _ in fresh]

    def advance(st):
        g, seed, _ = st
        Y, Z, X = g.shape
        orc.L.orc_run(g.ctypes.data, X, Y, Z, seed, 0, start, None, 1)
        st[2] = start

    t0 = time.perf_counter()
    run_parallel(advance, sorted(settled, key=lambda st: -st[0].size), threads)
    advance_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        oracle_rate(orc, settled, 0.5, threads, window=args.segment)
    vals = []
    for _ in range(args.steps):
        v, info = oracle_rate(orc, settled, args.cpu_budget / max(args.steps, 1), threads, window=args.segment)
        vals.append(v)
    v = float(np.mean(vals))
    vf, info_f = oracle_rate(orc, fresh, args.cpu_budget / 2, threads, window=args.segment)
    sample_txt = (f"{len(sample)} of the {args.worlds} worlds (every 16th), advanced untimed to step "
                  f"{start} ({advance_s:.1f} s), then their next {args.segment} steps, over and over, "
                  f"in 4-step takes for {args.cpu_budget:g} s over {args.steps} timed steps; {ORACLE_FLAGS}")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"batched: {args.worlds} mixed worlds (bounded CPU sample), the states from "
                                   f"step {start} on, as the GPU arm's timed segments",
                       "master_seed": args.master, "timed_from_step": start},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample_txt},
            "value_fresh": {"value": vf, "unit": UNIT,
                            "states": f"the same worlds freshly generated, their first {args.segment} steps",
                            "seconds": info_f["seconds"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU arm
def run_fs3d(args):
    import torch
    import fallingsand3d_gb300 as fs3d

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from fallingsand3d_gb300 import sharding
    master = sharding.weak_master(args.master, rank)  # weak scaling: each rank steps its own 2048-world batch
    worlds = batch_worlds(fs3d, master, args.worlds)
    cells = int(sum(X * Y * Z for (X, Y, Z), _ in worlds))
    shapes = [(Y, Z, X) for (X, Y, Z), _ in worlds]
    S = args.segment
    threads = os.cpu_count() or 1
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    if args.timed_from % S:
        raise SystemExit("--timed-from must be a multiple of --segment")

    # ---- headline: batched pool, device-resident
    host = gen_grids(fs3d, worlds, pinned_torch=torch)
    b = fs3d.Batch(150 << 30, steps_per_segment=S)
    # untimed: warm-up segments (the worlds leave their first steps, the phase
    # where everything still falls), the launch configuration chosen on real
    # segments, then plain segments up to where the timed segments start (the
    # reference arm steps the same states)
    pre = max(args.warmup, 3)
    untimed = untimed_segments(args)
    total_steps = S * (untimed + args.steps + 1 + 32)
    tickets = [b.admit(g.numpy(), seed, total_steps) for g, (_, seed) in zip(host, worlds)]
    bstream = torch.cuda.ExternalStream(b.stream())
    for _ in range(pre):
        b.run_segment()
    # two timed segments per candidate (the fastest counts): one alone let the
    # segment-to-segment spread pick the slower promotion now and then
    tune = b.autotune(trial_segments=2) if not args.no_autotune else {"segments": 0}
    done_untimed = pre + tune["segments"]
    if tune["segments"] not in (0, TUNE_SEGMENTS):
        raise RuntimeError(f"the autotuner ran {tune['segments']} segments, not {TUNE_SEGMENTS}: "
                           "the reference arm would step other states")
    for _ in range(untimed - done_untimed):
        b.run_segment()
    b.sync()
    checks = OracleChecks() if rank == 0 and not args.no_check else None
    # the worlds' states before the last timed segment (read back untimed):
    # the oracle checks that segment for every world
    before = pinned_views(torch, shapes) if checks is not None else None
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    seg_ms = []
    ctr0 = b.counters()
    launches0 = fs3d.kernel_launches()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            if before is not None and k == args.steps - 1:
                launches_snap = fs3d.kernel_launches()
                b.read_many(tickets, [v.data_ptr() for v in before])
                launches0 += fs3d.kernel_launches() - launches_snap
            flush.fill_(1)  # L2 flush between timed segments (outside the events)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(bstream)
            b.run_segment()
            e1.record(bstream)
            e1.synchronize()
            seg_ms.append(e0.elapsed_time(e1))
    launches = fs3d.kernel_launches() - launches0
    torch.cuda.synchronize()
    ctr1 = b.counters()
    dense_cs = ctr1["dense_cell_steps"] - ctr0["dense_cell_steps"]
    proc_cs = ctr1["processed_cell_steps"] - ctr0["processed_cell_steps"]
    proc_frac = proc_cs / dense_cs if dense_cs else 1.0
    ms = float(np.mean(seg_ms))
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = cells * S * world / (ms / 1e3)
    T0 = S * (untimed + args.steps)  # the step the timed segments left the worlds at
    steady = pinned_views(torch, shapes)
    b.sync()
    b.retire_many(tickets, [v.data_ptr() for v in steady])
    b.close()
    if checks is not None:
        for i in range(len(worlds)):
            checks.add_run("last timed segment", before[i].numpy(), worlds[i][1], T0 - S, S, steady[i].numpy())
        for i in range(3):  # three worlds from their first step to the last
            checks.add_run("timed batch from step 0", host[i].numpy(), worlds[i][1], 0, T0, steady[i].numpy())

    # ---- fresh: the same worlds generated anew, one segment from step 0 (device-timed)
    fresh_ms, fresh_build_ms = [], []
    for rep in range(3 + args.steps):
        fb = fs3d.Batch(150 << 30, steps_per_segment=S)
        fstream = torch.cuda.ExternalStream(fb.stream())
        fts = [fb.admit_generated(X, Y, Z, seed, S) for (X, Y, Z), seed in worlds]
        fb.sync()
        # the 2048 new worlds' tables, built and uploaded before the timed
        # region (a server builds them while the previous segment runs)
        hb = time.perf_counter()
        fb.prepare()
        fresh_build_ms.append((time.perf_counter() - hb) * 1e3)
        fb.sync()
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(fstream)
        fb.run_segment()
        e1.record(fstream)
        e1.synchronize()
        if rep >= 3:
            fresh_ms.append(e0.elapsed_time(e1))
        fb.retire_many(fts)
        fb.close()
    fresh_seg_ms = float(np.mean(fresh_ms))

    # ---- e2e through the C ABI from pinned host buffers
    # one step = admit every world from pinned host memory (H2D + conversion),
    # one segment, retire every world into pinned host memory (conversion + D2H).
    # The inputs are the worlds as the timed segments left them (step T0), so
    # e2e and `value` step the same world states.  The grids sit back to back
    # in one page-locked arena (and so do the outputs), so each direction is
    # one copy-engine transfer over the host link.  Timed steps are pipelined
    # through the asynchronous calls, as a server runs them: step i+1's upload
    # is enqueued before step i's read-back and before segment i+1, so both
    # directions of the link overlap the segments; the clock stops when the
    # last step's grids are in host memory.  e2e_fresh: the same with the
    # freshly generated worlds at step 0 (everything still falling).
    h2d, d2h = cells, cells
    outs2 = [pinned_views(torch, shapes) for _ in range(2)]
    outs = outs2[0]
    seeds = np.array([seed for _, seed in worlds], dtype=np.uint64)
    dims_xyz = np.array([d for d, _ in worlds], dtype=np.int64)
    out_ptrs2 = [np.array([o.data_ptr() for o in ob], dtype=np.uint64) for ob in outs2]

    def e2e_run(inputs, start):
        """--e2e-batches batches take steps in turn (default 1; with 2, as a
        double-buffered server would, twice as many steps are in flight: a
        batch cannot take the next step's worlds before its segment is
        enqueued, since the segment would step them too)."""
        in_ptrs = np.array([g.data_ptr() for g in inputs], dtype=np.uint64)
        starts = np.full(len(worlds), start, dtype=np.uint64)
        seq = []
        nb = max(1, min(2, args.e2e_batches))
        ebs = [fs3d.Batch(150 << 30, steps_per_segment=S) for _ in range(nb)]
        try:
            # untimed warm-up (captures the segment graphs, grows the pools),
            # then two steps through the waiting calls, one after the other
            for it in range(4):
                eb = ebs[it % nb]
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                ts = eb.admit_many(None, seeds, S, start_steps=starts, ptrs=in_ptrs, dims=dims_xyz)
                eb.run_segment()
                eb.retire_many(ts, out_ptrs2[it % nb])
                seq.append((time.perf_counter() - t0) * 1e3)
            torch.cuda.synchronize()
            host = {"admit_many_async": 0.0, "retire_many_async": 0.0, "run_segment": 0.0}
            pc = time.perf_counter
            # three timed runs of e2e_steps pipelined steps each, the median
            # reported: one host hiccup in a 50 ms run would otherwise move it;
            # the interpreter's collector is held off while the clock runs
            runs = []
            gc.collect()
            gc.disable()
            try:
                for _ in range(3):
                    t0 = pc()
                    prev = [None] * nb
                    for it in range(args.e2e_steps):
                        k = it % nb
                        a = pc()
                        ts = ebs[k].admit_many(None, seeds, S, start_steps=starts, ptrs=in_ptrs, dims=dims_xyz,
                                               wait=False)
                        b_ = pc()
                        if prev[k] is not None:
                            ebs[k].retire_many(prev[k], out_ptrs2[k], wait=False)
                        c = pc()
                        ebs[k].run_segment()
                        host["admit_many_async"] += b_ - a
                        host["retire_many_async"] += c - b_
                        host["run_segment"] += pc() - c
                        prev[k] = ts
                    for k in range(nb):
                        if prev[k] is not None:
                            ebs[k].retire_many(prev[k], out_ptrs2[k], wait=False)
                    for eb in ebs:
                        eb.wait_copies()
                    runs.append((pc() - t0) * 1e3 / args.e2e_steps)
            finally:
                gc.enable()
            ms = float(np.median(runs))
        finally:
            for eb in ebs:
                eb.close()
        host_ms = {k: round(v * 1e3 / (3 * args.e2e_steps), 3) for k, v in host.items()}
        return ms, float(np.mean(seq[2:])), host_ms, [round(r, 3) for r in runs]

    # every output of a round trip is its input stepped S steps (each e2e
    # step admits the same inputs, so the arena holds that result): all
    # worlds are checked against the oracle
    fresh_e2e_ms, fresh_seq, fresh_host_ms, fresh_runs = e2e_run(host, 0)
    if checks is not None:
        for i in range(len(worlds)):
            checks.add_run("fresh e2e round trip", host[i].numpy(), worlds[i][1], 0, S, outs[i].numpy().copy())
    e2e_ms, seq_ms, e2e_host_ms, e2e_runs = e2e_run(steady, T0)
    if checks is not None:
        for i in range(len(worlds)):
            checks.add_run("e2e round trip", steady[i].numpy(), worlds[i][1], T0, S, outs[i].numpy().copy())
    e2e_val = cells * S / (e2e_ms / 1e3)

    # ---- plain per-world launches of the drop-in kernel: one launch per world
    # per step from native code (fs3d_step_device_many), on the same states
    # as the timed segments' (step T0), device-resident
    offs, off = [], 0
    for (X, Y, Z), _ in worlds:
        offs.append(off)
        off += (X * Y * Z + 255) // 256 * 256
    pool = torch.empty(off, dtype=torch.uint8, device=dev)
    for o, g in zip(offs, steady):
        pool[o:o + g.numel()].copy_(g.reshape(-1), non_blocking=True)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream(dev)
    sp = st.cuda_stream
    ptrs = [pool.data_ptr() + o for o in offs]
    wseeds = [seed for _, seed in worlds]
    wdims = [d for d, _ in worlds]
    fs3d.step_device_many(ptrs, wdims, wseeds, T0, 2, sp)  # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    fs3d.step_device_many(ptrs, wdims, wseeds, T0 + 2, S, sp)
    e1.record(st)
    e1.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_val = cells * S / (plain_ms / 1e3)
    del pool

    # ---- plain single world 512^3 (drop-in byte kernel, HBM-bound)
    p512 = None
    if not args.skip_512:
        X = Y = Z = 512
        g = fs3d.gen_pillars(1, X, Y, Z)
        d = torch.from_numpy(g).to(dev)
        fs3d.step_device(d.data_ptr(), X, Y, Z, 1, 0, 8, sp)
        torch.cuda.synchronize()
        n = 1000  # the pillar workload runs 1000 steps
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fs3d.step_device(d.data_ptr(), X, Y, Z, 1, 8, n, sp)
        e1.record(st)
        e1.synchronize()
        t512 = e0.elapsed_time(e1) / n
        hbm, src = peaks()
        gbs = 2.0 * X * Y * Z / (t512 / 1e3) / 1e9
        p512 = {"workload": "512^3 pillars, drop-in byte kernel, steps 8..1007 (1000 steps)", "us_per_step": round(t512 * 1e3, 2),
                "voxel_updates_per_s": X * Y * Z / (t512 / 1e3), "algorithmic_gbs": round(gbs, 1),
                "hbm_frac": round(gbs / hbm, 3), "peak_gbs": hbm, "peak_source": src,
                "note": "134 MB grid read+written per step, in place (comparable to the 126 MB L2): the "
                        "algorithmic figure counts 2 B per cell; dram_* are the DRAM bytes ncu measured"}
        warm = profile_values("k_step_rows64_pillars512_warm", ("dram_bytes_per_launch", "duration_ns"))
        if warm:
            dram_gbs = warm["dram_bytes_per_launch"] / warm["duration_ns"]
            p512.update({"dram_gbs": round(dram_gbs, 1), "dram_frac": round(dram_gbs / hbm, 3),
                         "dram_source": "ncu, 3 warm launches at steps ~990 (profiles/k_step_rows64_pillars512_warm.md)"})
        # same world through the plane layout (the per-step kernel that skips settled row-pairs)
        with fs3d.World(g, 1, 0, fs3d.LAYOUT_PLANES) as w:
            w.step(8)
            ws = torch.cuda.ExternalStream(w.stream())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ws)
            w.step(n)
            e1.record(ws)
            e1.synchronize()
            tp = e0.elapsed_time(e1) / n
        p512["planes_us_per_step"] = round(tp * 1e3, 2)
        p512["planes_voxel_updates_per_s"] = X * Y * Z / (tp / 1e3)
        del d

    # ---- served: Poisson request streams through the continuous-batching loop
    served = None
    if not args.skip_serve:
        served = {}

        def serve_one(lam, seconds, **kw):
            p = fs3d.serve_params(lam, seconds, master_seed=args.master + 100, **kw)
            st_, reqs = fs3d.serve(p)
            wait = np.array([(r.admitted_s - r.arrival_s) * 1e3 for r in reqs]) if reqs else np.zeros(1)
            return {"requests": st_["requests"], "completed": st_["completed"], "p50_ms": round(st_["p50_ms"], 3),
                    "admission_wait_ms_p50_p99": [round(float(np.percentile(wait, 50)), 3),
                                                  round(float(np.percentile(wait, 99)), 3)],
                    "p99_ms": round(st_["p99_ms"], 3), "max_ms": round(st_["max_ms"], 3),
                    "voxel_updates_per_s": st_["voxel_updates_per_s"],
                    "offered_voxel_updates_per_s": st_["offered_voxel_updates_per_s"],
                    "served_fraction_of_offered": round(st_["voxel_updates_per_s"] /
                                                        max(st_["offered_voxel_updates_per_s"], 1.0), 3),
                    "peak_live_worlds": st_["peak_live_worlds"], "peak_bytes": st_["peak_bytes"],
                    "segments": st_["segments"], "wall_s": round(st_["wall_s"], 3)}

        for lam in (500.0, 2000.0, 8000.0):
            served[str(int(lam))] = serve_one(lam, args.serve_seconds)
        # past the headline rates, until the loop no longer keeps up: the
        # served rate falls below the offered one and the latency grows
        sweep = {}
        for lam in (32000.0, 64000.0, 128000.0):
            sweep[str(int(lam))] = serve_one(lam, args.serve_seconds / 5)
        served["saturation"] = sweep
        # a budget that binds: 2 MiB of pool for 8000 req/s, where the live
        # worlds want about 6 MB at their peak (the 150 GiB pool holds about
        # 300 000 of the largest requests, so at these request sizes it never
        # binds): arrivals wait for memory, results stay exact
        served["budget_2MiB_8000"] = serve_one(8000.0, args.serve_seconds / 2.5, hbm_budget=2 << 20)
        served["config"] = (f"{args.serve_seconds:g} s of arrivals per headline rate ({args.serve_seconds / 5:g} s "
                            f"for the saturation sweep, {args.serve_seconds / 2.5:g} s for the tight budget); dims iid "
                            "from {16..128}^3, n_steps "
                            "log-uniform in [10, 1000], 150 GiB budget unless stated, 64-step segments; latency = "
                            "arrival to hash visible on the host")

    # ---- large world + render: 1024^3 dunes, every step followed by a 1920x1080 DDA frame
    large = None
    if not args.skip_large:
        large = run_large(fs3d, torch, dev, args, checks)

    # ---- mesh materials: the upstream cube-grid scene
    mesh = None if args.skip_large else run_mesh(fs3d, torch, args, checks)

    # ---- an engine's frame loop: the 64^3 parity world, one step per call
    engine = run_engine_loop(fs3d, torch, checks)

    # ---- roofline of the dominant work: the segment graph, whose time is the
    # resident kernels (one launch per size class steps its worlds 64 times).
    # Algorithmic bytes = the 2-bit state read and written by every EVALUATED
    # cell-step (0.5 B each; layer pairs whose rows are settled are skipped
    # exactly and counted in the dense-equivalent figures only), per segment
    # with the events above; `traffic` = DRAM bytes per segment from the ncu
    # capture in profiles/.
    hbm, src = peaks()
    alg_bytes = 0.5 * cells * S * proc_frac
    achieved = alg_bytes / (ms / 1e3) / 1e9
    traffic, traffic_cells = profile_traffic("k_plane_segment_resident_batch2048")
    if traffic is not None and traffic_cells:
        traffic = traffic * cells / traffic_cells
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 3), "traffic": traffic,
                "kernel": "segment graph: k_plane_segment_resident (shared- and global-memory classes)",
                "launch": f"one {S}-step segment", "peak_source": src, "alg_bytes_per_launch": alg_bytes,
                "dense_equiv_state_gbs": round(0.5 * cells * S / (ms / 1e3) / 1e9, 1),
                "processed_fraction": round(proc_frac, 4),
                "note": "algorithmic bytes count the evaluated cell-steps (settled layer pairs are skipped "
                        "exactly); the worlds stay in L2, so DRAM sees a few MB per segment; the kernels are "
                        "latency-bound: each world's steps are a serial chain (see profiles/)"}
    # the issue-rate roof beside it: the warp instructions of one steady segment
    # (ncu, profiles/) against 4 issue slots per SM per cycle at the sampled clock
    clocks = clk.summary()
    inst = profile_values("k_plane_segment_resident_batch2048", ("warp_instructions_per_launch",))
    if inst is not None:
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        mhz = clocks.get("sm_mhz") or 2070.0
        issue_peak = sms * 4 * mhz * 1e6
        roofline["issue"] = {"warp_instructions_per_launch": inst["warp_instructions_per_launch"],
                             "achieved_per_s": round(inst["warp_instructions_per_launch"] / (ms / 1e3), 1),
                             "peak_per_s": issue_peak,
                             "frac": round(inst["warp_instructions_per_launch"] / (ms / 1e3) / issue_peak, 3),
                             "source": "ncu smsp__inst_executed.sum of one steady segment's launches; peak = "
                                       f"{sms} SMs x 4 issue slots x {mhz:.0f} MHz"}

    # ---- CPU leg (rank 0): the oracle timed (N=1) on the same world states
    # the GPU stepped, then the recorded GPU results checked against it
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        orc = load_oracle()
        idx = oracle_sample_index(len(worlds))
        if before is not None:
            settled = [[before[i].numpy().copy(), worlds[i][1], T0 - S] for i in idx]
            settled_txt = f"the states the last timed segment started from (step {T0 - S})"
        else:
            settled = [[steady[i].numpy().copy(), worlds[i][1], T0] for i in idx]
            settled_txt = f"the states the timed segments left (step {T0})"
        v, info = oracle_rate(orc, settled, args.cpu_budget, threads, window=S)
        fresh_states = [[host[i].numpy().copy(), worlds[i][1], 0] for i in idx]
        vf, info_f = oracle_rate(orc, fresh_states, args.cpu_budget / 2, threads, window=S)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{len(idx)} of the {args.worlds} worlds (every 16th), {settled_txt}, their next {S} "
                         f"steps over and over in 4-step takes for {info['seconds']} s; {ORACLE_FLAGS}",
               "fresh": {"value": vf, "unit": UNIT,
                         "states": f"the same worlds freshly generated, their first {S} steps over and over",
                         "seconds": info_f["seconds"]}}
    parity = None
    if checks is not None:
        res = checks.check(threads)
        parity = res["parity"]
        if large is not None and "large" in res:
            large.update(res["large"])
        if mesh is not None and "mesh" in res:
            mesh.update(res["mesh"])

    if rank == 0:
        fresh_value = cells * S / (fresh_seg_ms / 1e3)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u8", "data": "synthetic",
                "config": {"workload": f"batched: {args.worlds} worlds, dims iid from {{16,24,32,48,64,96,128}}^3, "
                                       f"{S}-step CUDA-graph segments (one step = one segment), timed from step "
                                       f"{S * untimed}",
                           "worlds_per_gpu": args.worlds, "cells_per_gpu": cells, "steps_per_segment": S,
                           "master_seed": args.master, "l2": "flushed between timed segments (512 MB write)",
                           "layout": "2-bit planes", "parallelism": f"replicas x{world}",
                           "launch_config": {k: tune.get(k) for k in ("mode", "promote", "ctas_per_sm", "trials")},
                           "timed_from_step": S * untimed, "untimed_segments": untimed},
                "gpu_launches": launches, "clocks": clocks, "roofline": roofline, "cpu_baseline": cpu,
                "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "ms": round(e2e_ms, 2), "steps": args.e2e_steps, "ms_runs": e2e_runs,
                        "timing": "median of three runs of the steps, each timed on the host from the first "
                                  "call to fs3d_batch_wait_copies returning",
                        "inputs": f"the {len(worlds)} worlds as the timed segments left them (step {T0}), "
                                  f"admitted at that step every e2e step",
                        "path": "fs3d_batch_admit_many_async (pinned arena) + fs3d_batch_run_segment + "
                                "fs3d_batch_retire_many_async (pinned arena), pipelined; fs3d_batch_wait_copies "
                                "at the end",
                        "batches": max(1, min(2, args.e2e_batches)),
                        "sequential_ms": round(seq_ms, 2),
                        "sequential_path": "fs3d_batch_admit_many + fs3d_batch_run_segment + fs3d_batch_retire_many, "
                                           "each step waited for",
                        "host_ms_per_step": e2e_host_ms},
                "value_fresh": {"value": fresh_value, "unit": UNIT, "ms_per_segment": round(fresh_seg_ms, 4),
                                "states": "the same worlds freshly generated (device), one segment from step 0; "
                                          "the segment's tables built beforehand (fs3d_batch_prepare, host time "
                                          "below); L2 flushed before each",
                                "table_build_host_ms": round(float(np.mean(fresh_build_ms[3:])), 3),
                                "vs_cpu_fresh": round(fresh_value / cpu["fresh"]["value"], 1) if cpu else None},
                "e2e_fresh": {"value": cells * S / (fresh_e2e_ms / 1e3), "unit": UNIT, "ms": round(fresh_e2e_ms, 2),
                              "ms_runs": fresh_runs,
                              "sequential_ms": round(fresh_seq, 2), "host_ms_per_step": fresh_host_ms,
                              "inputs": "the freshly generated worlds at step 0 (everything still falling), "
                                        "same calls and pipelining",
                              "vs_cpu_fresh": round(cells * S / (fresh_e2e_ms / 1e3) / cpu["fresh"]["value"], 1)
                              if cpu else None},
                "plain_per_world": {"value": plain_val, "unit": UNIT, "ms_per_segment": round(plain_ms, 2),
                                    "launches_per_segment": S * len(worlds),
                                    "us_per_launch": round(plain_ms * 1e3 / (S * len(worlds)), 2),
                                    "path": "fs3d_step_device_many: one launch of the drop-in kernel per world per "
                                            "step from native code, the timed segments' world states",
                                    "speedup_batched_vs_plain": round(value / world / plain_val, 2)},
                "processed": {"voxel_updates_per_s": value * proc_frac, "fraction_of_dense": round(proc_frac, 4),
                              "note": "value counts every cell of every world each step (dense-equivalent); "
                                      "this counts the cell-steps the kernels evaluated"},
                "plain_512": p512, "served": served, "large_render": large, "mesh_render": mesh, "engine_loop": engine, "parity": parity,
                "segment_ms": [round(x, 4) for x in seg_ms], "fresh_segment_ms": [round(x, 4) for x in fresh_ms]}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_large(fs3d, torch, dev, args, checks=None, X=1024, Y=1024, Z=1024, W=1920, H=1080):
    """1024^3 dune world (plane layout, per-step kernel), each step followed by
    a 1920x1080 DDA frame into a device buffer; per-material mass is checked
    against the initial grid, and the last frame is recorded in `checks` for
    the CPU DDA."""
    g = fs3d.gen_dunes(1, X, Y, Z)
    counts0 = np.bincount(g.reshape(-1), minlength=4)
    cam = fs3d.camera_world_view(X, Y, Z, W, H)
    frame = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    with fs3d.World(g, 1, 0, fs3d.LAYOUT_PLANES) as w:
        ws = torch.cuda.ExternalStream(w.stream())
        for _ in range(3):  # warm-up
            w.render(cam, W, H, fs3d.RENDER_DDA, out_ptr=frame.data_ptr())
        w.sync()
        n = args.large_steps
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        step_ms = frame_ms = 0.0
        t0 = time.perf_counter()
        for s in range(n):
            ev[0].record(ws)
            w.step(1)
            ev[1].record(ws)
            w.render(cam, W, H, fs3d.RENDER_DDA, out_ptr=frame.data_ptr())
            ev[2].record(ws)
            if s % 50 == 49 or s == n - 1:
                ev[2].synchronize()
            step_ms += ev[0].elapsed_time(ev[1]) if s % 50 == 49 else 0.0
            frame_ms += ev[1].elapsed_time(ev[2]) if s % 50 == 49 else 0.0
        w.sync()
        wall = time.perf_counter() - t0
        sampled = max(1, n // 50)
        last = frame.cpu().numpy()
        final = w.read()
    if checks is not None:
        checks.dda = (final, cam, W, H, last, 1e-5)
    counts = np.bincount(final.reshape(-1), minlength=4)
    cells = X * Y * Z
    return {"workload": f"{X}x{Y}x{Z} dunes (plane layout), {n} steps, each followed by a {W}x{H} fp32 DDA frame",
            "wall_s": round(wall, 3), "step_us": round(step_ms / sampled * 1e3, 2),
            "frame_us": round(frame_ms / sampled * 1e3, 2),
            "voxel_updates_per_s": cells * n / wall, "rays_per_s": W * H * n / wall,
            "mass_conserved": bool((counts == counts0).all())}


def run_engine_loop(fs3d, torch, checks=None, steps=200):
    """The drop-in use of an engine's main loop (upstream engine.cpp:54-74):
    the 64^3 parity world (two stone layers, sand and water in the upper
    half) stepped one step per call, as a frame loop would.  The world fits
    one CTA's shared memory and keeps its layer flags from call to call.
    Device time per call with CUDA events on the world's stream, and the
    host's time per call; the final grid is checked against the oracle."""
    g = fs3d.gen_parity(1)
    with fs3d.World(g, 1, 0, fs3d.LAYOUT_PLANES) as w:
        ws = torch.cuda.ExternalStream(w.stream())
        for _ in range(5):
            w.step(1)
        w.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(ws)
        for _ in range(steps):
            w.step(1)
        e1.record(ws)
        host_s = time.perf_counter() - t0
        e1.synchronize()
        final = w.read()
    if checks is not None:
        checks.add_run("engine loop", g, 1, 0, 5 + steps, final)
    dev_ms = e0.elapsed_time(e1)
    return {"workload": f"64^3 parity world, {steps} calls of one step each (steps 5..{4 + steps})",
            "us_per_step": round(dev_ms * 1e3 / steps, 2), "host_us_per_call": round(host_s * 1e6 / steps, 2),
            "voxel_updates_per_s": 64 ** 3 * steps / (dev_ms / 1e3)}


def run_mesh(fs3d, torch, args, checks=None, W=1920, H=1080, frames=20):
    """The cube-grid scene of the upstream renderer (renderer.cpp:1328-1352):
    51 x 51 green cubes (basic_mat) at y = 0 and 51 x 51 red textured cubes
    (textured_mat) at y = 5, each 0.2 in scale, one draw per cube; a seeded
    512 x 512 texture stands in for the texture file.  Frame time with CUDA
    events; the last frame is recorded in `checks` for the CPU restatement."""
    f = fs3d.mesh_cube().reshape(-1, 3)
    cube = np.c_[f, (f[:, [0, 2]] + 1) * 0.5].astype(np.float32)
    rng = np.random.default_rng(2024)
    tex = rng.integers(0, 256, (512, 512, 4), dtype=np.uint8)
    dv, dt = torch.from_numpy(cube).cuda(), torch.from_numpy(tex).cuda()
    gpu, cpu = [], []
    for y, mat, col in ((0.0, fs3d.MAT_BASIC, (0.0, 1.0, 0.0, 1.0)), (5.0, fs3d.MAT_TEXTURED, (1.0, 0.0, 0.0, 1.0))):
        for x in range(-25, 26):
            for z in range(-25, 26):
                m = np.diag([0.2, 0.2, 0.2, 1.0])
                m[:3, 3] = (x, y, z)
                gpu.append(fs3d.mesh_draw(dv.data_ptr(), 36, mat, m, col, dt.data_ptr() if mat else 0, 512, 512))
                cpu.append(dict(vertices=cube, material=mat, model=m, color=col, texture=tex if mat else None))
    kw = dict(cam_pos=(0.0, -4.0, -32.0), rot_y=0.0)
    view = fs3d.object_view_scene(**kw)
    gpu = fs3d.mesh_draws(gpu)
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    for _ in range(3):
        fs3d.render_meshes_device(view, gpu, W, H, out.data_ptr(), st.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(frames):
        fs3d.render_meshes_device(view, gpu, W, H, out.data_ptr(), st.cuda_stream)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / frames
    got = out.cpu().numpy()
    if checks is not None:
        checks.mesh = (kw, cpu, W, H, got)
    return {"workload": f"{len(gpu)} cube draws ({12 * len(gpu)} triangles, basic_mat and textured_mat) at {W}x{H}",
            "frame_us": round(ms * 1e3, 1), "triangles_per_s": 12 * len(gpu) / (ms / 1e3),
            "pixels_covered": int((got != np.float32([0, 0, 1, 1])).any(-1).sum())}


def run_only(args):
    """One workload without the side measurements, for ncu captures:
    `batched` runs warmup + steps segments of the 2048-world pool, `plain512`
    runs warmup + steps x 8 steps of the drop-in byte kernel on 512^3, `large`
    runs the 1024^3 dune world with a 1920x1080 frame after each of
    --large-steps steps, `fresh` runs one segment of the 2048 freshly
    generated worlds, `e2e` reads the pool back after 20 segments and runs
    --e2e-steps pipelined e2e steps on those world states (after 3 waited-for
    warm-up steps)."""
    import torch
    import fallingsand3d_gb300 as fs3d
    if args.only == "fresh":
        # one segment of the freshly generated worlds (everything still falling)
        worlds = batch_worlds(fs3d, args.master, args.worlds)
        host = gen_grids(fs3d, worlds, pinned_torch=torch)
        seeds = np.array([sd for _, sd in worlds], dtype=np.uint64)
        dims = np.array([d for d, _ in worlds], dtype=np.int64)
        ptrs = np.array([g.data_ptr() for g in host], dtype=np.uint64)
        with fs3d.Batch(150 << 30, steps_per_segment=args.segment) as b:
            ts = b.admit_many(None, seeds, args.segment, ptrs=ptrs, dims=dims)
            b.run_segment()
            b.retire_many(ts)
        print(json.dumps({"only": args.only, "ok": True}))
        return 0
    if args.only == "e2e":
        worlds = batch_worlds(fs3d, args.master, args.worlds)
        S = args.segment
        shapes = [(Y, Z, X) for (X, Y, Z), _ in worlds]
        steady, outs = pinned_views(torch, shapes), pinned_views(torch, shapes)
        with fs3d.Batch(150 << 30, steps_per_segment=S) as b:
            ts = [b.admit_generated(X, Y, Z, seed, S * 20) for (X, Y, Z), seed in worlds]
            for _ in range(20):
                b.run_segment()
            b.retire_many(ts, [v.data_ptr() for v in steady])
        seeds = np.array([sd for _, sd in worlds], dtype=np.uint64)
        dims = np.array([d for d, _ in worlds], dtype=np.int64)
        inp = np.array([g.data_ptr() for g in steady], dtype=np.uint64)
        outp = np.array([o.data_ptr() for o in outs], dtype=np.uint64)
        starts = np.full(len(worlds), S * 20, dtype=np.uint64)
        with fs3d.Batch(150 << 30, steps_per_segment=S) as eb:
            for _ in range(3):
                t = eb.admit_many(None, seeds, S, start_steps=starts, ptrs=inp, dims=dims)
                eb.run_segment()
                eb.retire_many(t, outp)
            prev = None
            pc = time.perf_counter
            host = [0.0, 0.0, 0.0]
            torch.cuda.synchronize()
            t0 = pc()
            for _ in range(args.e2e_steps):
                a = pc()
                t = eb.admit_many(None, seeds, S, start_steps=starts, ptrs=inp, dims=dims, wait=False)
                b_ = pc()
                if prev is not None:
                    eb.retire_many(prev, outp, wait=False)
                c = pc()
                eb.run_segment()
                host[0] += b_ - a
                host[1] += c - b_
                host[2] += pc() - c
                prev = t
            eb.retire_many(prev, outp, wait=False)
            eb.wait_copies()
            ms = (pc() - t0) * 1e3 / args.e2e_steps
        n = args.e2e_steps
        print(json.dumps({"only": args.only, "ok": True, "ms_per_step": round(ms, 3),
                          "host_ms_per_step": {"admit_many_async": round(host[0] * 1e3 / n, 3),
                                               "retire_many_async": round(host[1] * 1e3 / n, 3),
                                               "run_segment": round(host[2] * 1e3 / n, 3)}}))
        return 0
    if args.only == "dunes":
        # the 1024^3 dune world stepped alone (no frames): per-step times over the run
        g = fs3d.gen_dunes(1, 1024, 1024, 1024)
        with fs3d.World(g, 1, 0, fs3d.LAYOUT_PLANES) as w:
            ws = torch.cuda.ExternalStream(w.stream())
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.large_steps + 1)]
            ev[0].record(ws)
            for s in range(args.large_steps):
                w.step(1)
                ev[s + 1].record(ws)
            ev[-1].synchronize()
            us = [ev[s].elapsed_time(ev[s + 1]) * 1e3 for s in range(args.large_steps)]
        marks = {str(a): round(float(np.mean(us[a:a + 10])), 1) for a in range(0, args.large_steps, 50)}
        print(json.dumps({"only": args.only, "ok": True, "mean_step_us": round(float(np.mean(us)), 2),
                          "step_us_by_step": marks}))
        return 0
    if args.only == "large":
        out = run_large(fs3d, torch, torch.device("cuda", 0), args)
        print(json.dumps({"only": args.only, "ok": True, "large_render": out}))
        return 0
    if args.only == "mesh":
        print(json.dumps({"only": args.only, "ok": True, "mesh_render": run_mesh(fs3d, torch, args)}))
        return 0
    if args.only == "batched":
        worlds = batch_worlds(fs3d, args.master, args.worlds)
        with fs3d.Batch(150 << 30, steps_per_segment=args.segment) as b:
            for (X, Y, Z), seed in worlds:
                b.admit_generated(X, Y, Z, seed, args.segment * (args.warmup + args.steps + 8))
            for _ in range(args.warmup):
                b.run_segment()
            tune = {"segments": 0}
            if not args.no_autotune:
                tune = b.autotune(trial_segments=2)  # as the headline run does before its timed segments
            for _ in range(args.steps):
                b.run_segment()
            b.sync()
        # segments run in all (a profiler selects the last one's class launches by this count)
        extra = {"segments": args.warmup + tune["segments"] + args.steps,
                 "tune": {k: tune.get(k) for k in ("mode", "promote", "ctas_per_sm")}}
    elif args.only == "plain512p":
        # the same world in the plane layout (per-step plane kernel), 8 steps per warm-up/step
        g = fs3d.gen_pillars(1, 512, 512, 512)
        with fs3d.World(g, 1, 0, fs3d.LAYOUT_PLANES) as w:
            w.step(8 * (args.warmup + args.steps))
            w.sync()
    else:
        g = fs3d.gen_pillars(1, 512, 512, 512)
        d = torch.from_numpy(g).cuda()
        fs3d.step_device(d.data_ptr(), 512, 512, 512, 1, 0, 8 * (args.warmup + args.steps),
                         torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
    print(json.dumps({"only": args.only, "ok": True, **(extra if args.only == "batched" else {})}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--e2e-steps", type=int, default=60, help="timed steps of the e2e leg (each of its three timed runs)")
    ap.add_argument("--e2e-batches", type=int, default=1, help="batches taking the e2e steps in turn (1 or 2)")
    ap.add_argument("--impl", default="fs3d", choices=["fs3d", "reference"])
    ap.add_argument("--worlds", type=int, default=2048)
    ap.add_argument("--master", type=int, default=1)
    ap.add_argument("--segment", type=int, default=64)
    ap.add_argument("--timed-from", type=int, default=640,
                    help="step at which the timed segments start (both arms step the states from there)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--skip-512", action="store_true")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--skip-large", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=5.0)
    ap.add_argument("--large-steps", type=int, default=500)
    ap.add_argument("--only", default="all", choices=["all", "batched", "plain512", "plain512p", "large", "dunes", "mesh", "e2e", "fresh"],
                    help="run one workload alone (profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.only != "all":
        return run_only(args)
    return run_fs3d(args)


if __name__ == "__main__":
    sys.exit(main())
