"""GPU checks of the batched / served path: many mixed-size worlds in one
pool, stepped in graph-captured segments, each bit-exact to the oracle and
identical whether run alone or inside any mix (continuous admission)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GiB = 1 << 30


def small_batch(fs3d, master, count, max_dim=64):
    dims, seeds = fs3d.gen_batch_dims(master, count)
    dims = np.minimum(dims, max_dim)
    return [(tuple(int(v) for v in dims[w]), int(seeds[w])) for w in range(count)]


def oracle_final(orc, fs3d, dims, seed, n, start=0):
    X, Y, Z = dims
    g = fs3d.gen_batch_world(seed, X, Y, Z)
    orc.run(g, seed, start, n, nthreads=0)
    return g


@pytest.mark.parametrize("use_graphs,use_smem", [(True, True), (False, True), (True, False), (False, False),
                                                  (True, 2), (False, 2)])
def test_batch_matches_oracle(fs3d, orc, use_graphs, use_smem):
    worlds = small_batch(fs3d, 5, 24, max_dim=128)
    rng = np.random.default_rng(1)
    steps = [int(v) for v in rng.integers(1, 150, len(worlds))]
    with fs3d.Batch(4 * GiB, steps_per_segment=64, use_graphs=use_graphs, use_smem=use_smem) as b:
        tickets = []
        for (dims, seed), n in zip(worlds, steps):
            X, Y, Z = dims
            tickets.append(b.admit(fs3d.gen_batch_world(seed, X, Y, Z), seed, n))
        for _ in range((max(steps) + 63) // 64):
            b.run_segment()
        b.sync()
        for t, (dims, seed), n in zip(tickets, worlds, steps):
            done, h = b.poll(t)
            assert done
            X, Y, Z = dims
            exp = oracle_final(orc, fs3d, dims, seed, n)
            assert h == orc.hash(exp), (dims, seed, n)
            got = b.retire(t, (Y, Z, X))
            assert (got == exp).all()
        assert b.stats()["live_worlds"] == 0 and b.stats()["bytes_used"] == 0


def test_mix_equals_alone_with_continuous_admission(fs3d, orc):
    worlds = small_batch(fs3d, 77, 30, max_dim=96)
    n = 100
    # alone: each world in its own batch
    alone = {}
    for dims, seed in worlds[:6]:
        X, Y, Z = dims
        with fs3d.Batch(GiB, steps_per_segment=32) as b:
            t = b.admit(fs3d.gen_batch_world(seed, X, Y, Z), seed, n)
            for _ in range(4):
                b.run_segment()
            b.sync()
            alone[seed] = b.poll(t)[1]
    # mix: worlds arrive while others are mid-flight, with a start step offset
    with fs3d.Batch(GiB, steps_per_segment=32) as b:
        live = {}
        pending = list(worlds)
        results = {}
        seg = 0
        while pending or live:
            for _ in range(3):
                if pending:
                    dims, seed = pending.pop(0)
                    X, Y, Z = dims
                    live[b.admit(fs3d.gen_batch_world(seed, X, Y, Z), seed, n)] = (dims, seed)
            b.run_segment()
            seg += 1
            for t in list(live):
                done, h = b.poll(t)
                if done:
                    results[live.pop(t)[1]] = h
                    b.retire(t)
            assert seg < 100
    for seed, h in alone.items():
        assert results[seed] == h
    for dims, seed in worlds[6:12]:
        assert results[seed] == orc.hash(oracle_final(orc, fs3d, dims, seed, n))


def test_budget_admission_and_release(fs3d):
    g = fs3d.gen_batch_world(1, 64, 64, 64)
    per = 64 * 64 * 16 + 64 + 64  # planes (64 x 64 rows of 16 bytes), layer flags (64 bytes), descriptor
    with fs3d.Batch(2 * per + 10, steps_per_segment=8) as b:
        t1 = b.admit(g, 1, 8)
        t2 = b.admit(g, 2, 8)
        assert b.try_admit(g, 3, 8) is None
        with pytest.raises(fs3d.Fs3dError) as e:
            b.admit(g, 3, 8)
        assert e.value.status == fs3d.ERR_BUDGET
        b.run_segment()
        b.retire(t1)
        t3 = b.admit(g, 3, 8)
        b.run_segment()
        b.sync()
        assert b.poll(t2)[0] and b.poll(t3)[0]
        with pytest.raises(fs3d.Fs3dError):
            b.poll(t1)


def test_start_step_offsets_parity(fs3d, orc):
    dims, seed = (48, 40, 24), 1234
    X, Y, Z = dims
    g = fs3d.gen_batch_world(seed, X, Y, Z)
    with fs3d.Batch(GiB, steps_per_segment=16) as b:
        t = b.admit(g, seed, 37, start_step=11)
        for _ in range(3):
            b.run_segment()
        b.sync()
        h = b.poll(t)[1]
    ref = g.copy()
    orc.run(ref, seed, 11, 37, nthreads=0)
    assert h == orc.hash(ref)


def test_device_generated_worlds_match_host_generator(fs3d, orc):
    dims, seeds = fs3d.gen_batch_dims(31, 12)
    with fs3d.Batch(GiB, steps_per_segment=16) as b:
        for w in range(12):
            X, Y, Z = (int(v) for v in dims[w])
            seed = int(seeds[w])
            t0 = b.admit_generated(X, Y, Z, seed, 0)
            assert (b.retire(t0, (Y, Z, X)) == orc.gen_c3_world(seed, X, Y, Z)).all(), (X, Y, Z)
        X, Y, Z = (int(v) for v in dims[0])
        t = b.admit_generated(X, Y, Z, int(seeds[0]), 40)
        for _ in range(3):
            b.run_segment()
        b.sync()
        ref = orc.gen_c3_world(int(seeds[0]), X, Y, Z)
        orc.run(ref, int(seeds[0]), 0, 40, nthreads=0)
        assert b.poll(t)[1] == orc.hash(ref)


def test_admit_many_and_retire_many(fs3d, orc):
    worlds = small_batch(fs3d, 17, 40, max_dim=96)
    grids = [fs3d.gen_batch_world(seed, *dims) for dims, seed in worlds]
    n = 70
    with fs3d.Batch(GiB, steps_per_segment=64) as b:
        tickets = b.admit_many(grids, [s for _, s in worlds], n)
        assert len(tickets) == len(worlds)
        for _ in range(2):
            b.run_segment()
        outs = [np.empty_like(g) for g in grids]
        b.retire_many(tickets, [o.ctypes.data for o in outs])
        assert b.stats()["live_worlds"] == 0
    for (dims, seed), g, o in list(zip(worlds, grids, outs))[:8]:
        ref = g.copy()
        orc.run(ref, seed, 0, n, nthreads=0)
        assert (o == ref).all()
    with fs3d.Batch(2 * (64 * 64 * 16 + 64 + 64) + 100, steps_per_segment=8) as b:
        big = [fs3d.gen_batch_world(1, 64, 64, 64)] * 3
        assert len(b.admit_many(big, [1, 2, 3], 8)) == 2  # the third does not fit


# dims that land in each resident class (one CTA of 128/256/768 threads,
# clusters of 2/4/8 CTAs) and one too large to be resident
CLASS_DIMS = [(16, 16, 16), (64, 64, 64), (64, 96, 128), (96, 96, 96), (128, 128, 128), (128, 256, 128),
              (64, 512, 128), (40, 37, 21), (130, 66, 90)]


@pytest.mark.parametrize("use_smem", [True, False, 2])
def test_every_resident_class_matches_oracle(fs3d, orc, use_smem):
    n = 67  # odd and not a multiple of the segment: phases and partial segments
    with fs3d.Batch(8 * GiB, steps_per_segment=32, use_smem=use_smem) as b:
        tickets = []
        for w, (X, Y, Z) in enumerate(CLASS_DIMS):
            g = fs3d.gen_batch_world(1000 + w, X, Y, Z)
            tickets.append((b.admit(g, 1000 + w, n, start_step=w), g))
        for _ in range(3):
            b.run_segment()
        b.sync()
        for w, ((t, g), dims) in enumerate(zip(tickets, CLASS_DIMS)):
            ref = g.copy()
            orc.run(ref, 1000 + w, w, n, nthreads=0)
            assert b.poll(t)[1] == orc.hash(ref), dims


@pytest.mark.parametrize("dims", CLASS_DIMS[:6])
def test_world_resident_path_matches_oracle(fs3d, orc, dims):
    X, Y, Z = dims
    g = fs3d.gen_batch_world(7, X, Y, Z)
    with fs3d.World(g, 7, 3, fs3d.LAYOUT_PLANES) as w:
        w.step(45)
        w.step(1)
        ref = g.copy()
        orc.run(ref, 7, 3, 46, nthreads=0)
        got = w.read()
    assert (got == ref).all()


def test_autotune_keeps_results_exact(fs3d, orc):
    """Tuning runs real segments under every candidate configuration (class
    promotion, per-step grid); the worlds must end exactly where the oracle
    puts them, and a second batch of the same make-up reuses the choice."""
    worlds = small_batch(fs3d, 21, 20, max_dim=160)
    worlds += [((300, 40, 96), 991), ((512, 64, 256), 992), ((2048, 6, 4), 993)]  # cluster and per-step worlds
    n = 600
    for rep in range(2):
        with fs3d.Batch(4 * GiB, steps_per_segment=32) as b:
            tickets = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, n) for dims, seed in worlds]
            rpt = b.autotune(trial_segments=1)
            assert rpt["cached"] == (rep == 1), rpt
            if rep == 0:
                assert rpt["trials"] >= 2 and rpt["best_vox_per_ms"] > 0, rpt
            assert 0 <= rpt["promote"] <= 2 and rpt["ctas_per_sm"] >= 1
            for _ in range(n // 32 + 1):
                b.run_segment()
            b.sync()
            for t, (dims, seed) in zip(tickets, worlds):
                done, h = b.poll(t)
                assert done
                exp = oracle_final(orc, fs3d, dims, seed, n)
                assert h == orc.hash(exp), (rep, dims, seed, rpt)


@pytest.mark.parametrize("dims", [CLASS_DIMS[0], CLASS_DIMS[2], CLASS_DIMS[3], CLASS_DIMS[5]])
@pytest.mark.parametrize("start", [0, 250, (1 << 32) - 7])
def test_settled_row_skip_long_segments(fs3d, orc, dims, start):
    """Resident launches skip row pairs whose rows did not change in the two
    previous steps, tracked by the low 8 bits of the step.  Long launches (the
    step counter wraps those 8 bits several times, from starts on and off the
    wrap) let most of a world settle while water keeps moving; the result must
    be the oracle's, step for step in the hashes."""
    X, Y, Z = dims
    seed = 4242
    g = fs3d.gen_batch_world(seed, X, Y, Z)
    ref = g.copy()
    with fs3d.World(g, seed, start, fs3d.LAYOUT_PLANES) as w:
        for n in (700, 1, 2, 300):
            w.step(n)
            orc.run(ref, seed, start, n, nthreads=0)
            start += n
            assert w.hash() == orc.hash(ref), (dims, start)
        assert (w.read() == ref).all()


def test_counters_dense_and_processed(fs3d, orc):
    """dense = every cell of every world per step; processed <= dense, and
    below it once the worlds have settled (first two steps of each segment
    evaluate everything)."""
    worlds = small_batch(fs3d, 8, 10, max_dim=64)
    n = 512
    with fs3d.Batch(GiB, steps_per_segment=128) as b:
        tickets = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, n) for dims, seed in worlds]
        for _ in range(n // 128):
            b.run_segment()
        c = b.counters()
        assert c["dense_cell_steps"] == n * sum(X * Y * Z for (X, Y, Z), _ in worlds)
        assert 0 < c["processed_cell_steps"] < c["dense_cell_steps"]
        for t, (dims, seed) in zip(tickets[:4], worlds):
            assert b.poll(t)[1] == orc.hash(oracle_final(orc, fs3d, dims, seed, n))


@pytest.mark.parametrize("use_smem", [True, 2])
def test_kept_layer_flags_across_segments(fs3d, orc, use_smem):
    """The layer change flags persist between segments (the first two steps of
    a segment are not re-evaluated densely); worlds of every class, segments
    of several lengths, joined by late admissions, must follow the oracle."""
    worlds = [((16, 16, 16), 1), ((64, 64, 64), 2), ((96, 96, 96), 3), ((128, 128, 128), 4), ((40, 37, 21), 5),
              ((16, 256, 16), 6), ((2048, 8, 6), 7)]
    n = 333
    with fs3d.Batch(8 * GiB, steps_per_segment=37, use_smem=use_smem) as b:
        tickets = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, n) for dims, seed in worlds[:4]]
        for _ in range(3):
            b.run_segment()
        late = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, n, start_step=250) for dims, seed in worlds[4:]]
        for _ in range(n // 37 + 1):
            b.run_segment()
        b.sync()
        for t, (dims, seed) in zip(tickets, worlds[:4]):
            assert b.poll(t)[1] == orc.hash(oracle_final(orc, fs3d, dims, seed, n)), dims
        for t, (dims, seed) in zip(late, worlds[4:]):
            assert b.poll(t)[1] == orc.hash(oracle_final(orc, fs3d, dims, seed, n, start=250)), dims


def test_admit_and_retire_many_pinned_and_device(fs3d, orc, cuda):
    """Grids in page-locked host memory and in device memory are gathered and
    scattered by one copy kernel (no copy call per world); pageable ones take
    a copy each.  A mix of all three, odd sizes included, must round-trip and
    step exactly."""
    worlds = small_batch(fs3d, 23, 18, max_dim=96) + [((37, 21, 13), 901), ((5, 7, 3), 902)]
    grids = [fs3d.gen_batch_world(seed, *dims) if dims[1] >= 4 else orc.gen_c1(seed, *dims)
             for dims, seed in worlds]
    kinds = ["pinned", "device", "pageable"]
    srcs, ptrs = [], []
    for i, g in enumerate(grids):
        k = kinds[i % 3]
        if k == "pinned":
            t = cuda.from_numpy(g.copy()).pin_memory()
        elif k == "device":
            t = cuda.from_numpy(g.copy()).cuda()
        else:
            t = g.copy()
        srcs.append(t)
        ptrs.append(t.data_ptr() if k != "pageable" else t.ctypes.data)
    outs, out_ptrs = [], []
    for i, g in enumerate(grids):
        k = kinds[(i + 1) % 3]
        if k == "pinned":
            t = cuda.zeros(g.shape, dtype=cuda.uint8).pin_memory()
        elif k == "device":
            t = cuda.zeros(g.shape, dtype=cuda.uint8, device="cuda")
        else:
            t = np.zeros_like(g)
        outs.append(t)
        out_ptrs.append(t.data_ptr() if k != "pageable" else t.ctypes.data)
    cuda.cuda.synchronize()
    n = 90
    with fs3d.Batch(GiB, steps_per_segment=64) as b:
        ts = b.admit_many(grids, [s for _, s in worlds], n, ptrs=ptrs)
        assert len(ts) == len(worlds)
        for _ in range(2):
            b.run_segment()
        b.retire_many(ts, out_ptrs)
    for (dims, seed), g, o in zip(worlds, grids, outs):
        ref = g.copy()
        orc.run(ref, seed, 0, n, nthreads=0)
        got = o.cpu().numpy() if hasattr(o, "cpu") else o
        assert (got == ref).all(), dims


@pytest.mark.parametrize("where", ["pinned", "device"])
def test_admit_and_retire_many_contiguous_runs(fs3d, orc, cuda, where):
    """Worlds stored back to back in one arena go over in one copy per run;
    a gap (and a world whose size is not a multiple of 16) ends a run."""
    worlds = small_batch(fs3d, 29, 14, max_dim=64) + [((37, 21, 13), 903)] + small_batch(fs3d, 31, 6, max_dim=48)
    grids = [fs3d.gen_batch_world(seed, *dims) for dims, seed in worlds]
    sizes = [g.size for g in grids]
    gap = 48
    total = sum(sizes) + gap

    def arena():
        t = cuda.zeros(total, dtype=cuda.uint8)
        return t.pin_memory() if where == "pinned" else t.cuda()

    src, dst = arena(), arena()
    offs, off = [], 0
    for i, n in enumerate(sizes):
        if i == 7:
            off += gap  # a hole in the middle of a run
        offs.append(off)
        off += n
    flat = cuda.from_numpy(np.concatenate([g.reshape(-1) for g in grids]))
    for o, n, g in zip(offs, sizes, grids):
        src[o:o + n].copy_(cuda.from_numpy(g.reshape(-1)))
    cuda.cuda.synchronize()
    del flat
    n_steps = 70
    with fs3d.Batch(GiB, steps_per_segment=64) as b:
        ts = b.admit_many(None, [s for _, s in worlds], n_steps, ptrs=[src.data_ptr() + o for o in offs],
                          dims=[d for d, _ in worlds])
        for _ in range(2):
            b.run_segment()
        b.retire_many(ts, [dst.data_ptr() + o for o in offs])
    out = dst.cpu().numpy()
    for (dims, seed), g, o, n in zip(worlds, grids, offs, sizes):
        ref = g.copy()
        orc.run(ref, seed, 0, n_steps, nthreads=0)
        assert (out[o:o + n].reshape(g.shape) == ref).all(), dims


def test_handles_used_from_several_threads(fs3d, orc):
    """Different handles may be used concurrently: four threads, each with its
    own batch (and one with a plane world), step and read back at once."""
    import threading
    results, errors = {}, []

    def run(tid):
        try:
            worlds = small_batch(fs3d, 40 + tid, 6, max_dim=64)
            n = 80
            with fs3d.Batch(GiB, steps_per_segment=32) as b:
                ts = [b.admit(fs3d.gen_batch_world(s, *d), s, n) for d, s in worlds]
                for _ in range(3):
                    b.run_segment()
                b.sync()
                results[tid] = [(d, s, b.poll(t)[1]) for t, (d, s) in zip(ts, worlds)]
            if tid == 0:
                g = fs3d.gen_batch_world(99, 96, 40, 72)
                with fs3d.World(g, 99, 0, fs3d.LAYOUT_PLANES) as w:
                    w.step(50)
                    results["world"] = w.hash()
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(repr(e))

    th = [threading.Thread(target=run, args=(i,)) for i in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for tid in range(4):
        for dims, seed, h in results[tid]:
            assert h == orc.hash(oracle_final(orc, fs3d, dims, seed, 80)), (tid, dims)
    ref = fs3d.gen_batch_world(99, 96, 40, 72)
    orc.run(ref, 99, 0, 50, nthreads=0)
    assert results["world"] == orc.hash(ref)


def test_tables_reused_between_changes(fs3d, orc):
    """Segments of an unchanged batch launch on the device tables as the last
    segment advanced them; every change (a world admitted or retired, a world
    turning old in the hybrid mode, a last partial segment) rebuilds them.
    All worlds, including one retired mid-run, follow the oracle."""
    S = 16
    worlds = [((16, 16, 16), 11, 16 * 20), ((64, 48, 32), 12, 16 * 9 + 5), ((96, 96, 96), 13, 7),
              ((24, 128, 40), 14, 16 * 18), ((2048, 8, 6), 15, 16 * 12 + 3)]
    with fs3d.Batch(4 * GiB, steps_per_segment=S) as b:
        tickets = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, n) for dims, seed, n in worlds[:4]]
        early = b.admit(fs3d.gen_batch_world(21, 32, 32, 32), 21, 1000)
        for _ in range(5):
            b.run_segment()
        dims, seed, n = worlds[4]
        tickets.append(b.admit(fs3d.gen_batch_world(seed, *dims), seed, n, start_step=100))
        for _ in range(3):
            b.run_segment()
        X, Y, Z = 32, 32, 32
        got = b.retire(early, (Y, Z, X))
        assert (got == oracle_final(orc, fs3d, (32, 32, 32), 21, 8 * S)).all()
        for _ in range(20):
            b.run_segment()
        b.sync()
        for t, (dims, seed, n) in zip(tickets, worlds):
            done, h = b.poll(t)
            assert done, dims
            start = 100 if seed == 15 else 0
            assert h == orc.hash(oracle_final(orc, fs3d, dims, seed, n, start=start)), dims
        dense = b.counters()["dense_cell_steps"]
        assert dense == sum(X * Y * Z * n for (X, Y, Z), _, n in worlds) + 32 ** 3 * 8 * S


def _with_statics(fs3d, worlds, every=3):
    """Batch worlds; every `every`-th one also holds static materials (bytes
    >= 4), which stay in place and come back unchanged on read-back."""
    grids = []
    for i, (dims, seed) in enumerate(worlds):
        g = fs3d.gen_batch_world(seed, *dims)
        if i % every == 1:
            rng = np.random.default_rng(seed)
            idx = rng.integers(0, g.size, 64)
            g.reshape(-1)[idx] = rng.integers(4, 256, 64).astype(np.uint8)
        grids.append(g)
    return grids


def test_pipelined_async_admit_and_retire(fs3d, orc, cuda):
    """admit_many_async / retire_many_async pipelined on one batch the way a
    server overlaps the host link with compute: step i+1's uploads are
    enqueued before step i's read-backs and before segment i+1.  Worlds with
    static materials get their byte copies once their flags reach the host.
    Every output equals the oracle."""
    S = 32
    worlds = small_batch(fs3d, 41, 10, max_dim=64) + [((37, 21, 13), 904), ((5, 7, 3), 905)]
    grids = _with_statics(fs3d, worlds[:-1]) + [orc.gen_c1(905, 5, 7, 3)]
    sizes = [g.size for g in grids]
    offs = [int(v) for v in np.concatenate([[0], np.cumsum(sizes)[:-1]])]
    total = int(sum(sizes))
    src = cuda.from_numpy(np.concatenate([g.reshape(-1) for g in grids])).pin_memory()
    steps = 4
    outs = [cuda.zeros(total, dtype=cuda.uint8).pin_memory() for _ in range(steps)]
    seeds = [s for _, s in worlds]
    dims = [d for d, _ in worlds]
    with fs3d.Batch(GiB, steps_per_segment=S) as b:
        prev = None
        for i in range(steps):
            ts = b.admit_many(None, seeds, S, start_steps=[1000 * i] * len(worlds),
                              ptrs=[src.data_ptr() + o for o in offs], dims=dims, wait=False)
            assert len(ts) == len(worlds)
            if prev is not None:
                b.retire_many(prev[0], [outs[prev[1]].data_ptr() + o for o in offs], wait=False)
            b.run_segment()
            prev = (ts, i)
        b.retire_many(prev[0], [outs[prev[1]].data_ptr() + o for o in offs], wait=False)
        b.wait_copies()
        assert b.stats()["live_worlds"] == 0 and b.stats()["bytes_used"] == 0
    for i in range(steps):
        got = outs[i].numpy()
        for (d, seed), g, o, n in zip(worlds, grids, offs, sizes):
            ref = g.copy()
            orc.run(ref, seed, 1000 * i, S, nthreads=0)
            assert (got[o:o + n].reshape(g.shape) == ref).all(), (i, d)


def test_async_admission_poll_and_single_retire(fs3d, orc, cuda):
    """A world admitted without a host wait can be polled (its hash needs the
    static copy) and retired singly before any other call completes its
    admission; a synchronous admit_many of static worlds still reads back."""
    worlds = small_batch(fs3d, 43, 6, max_dim=48)
    grids = _with_statics(fs3d, worlds, every=2)
    pinned = [cuda.from_numpy(g.copy()).pin_memory() for g in grids]
    n = 40
    with fs3d.Batch(GiB, steps_per_segment=64) as b:
        ts = b.admit_many(None, [s for _, s in worlds], n, ptrs=[p.data_ptr() for p in pinned],
                          dims=[d for d, _ in worlds], wait=False)
        b.run_segment()
        b.sync()
        for t, (d, seed), g in zip(ts, worlds, grids):
            ref = g.copy()
            orc.run(ref, seed, 0, n, nthreads=0)
            done, h = b.poll(t)
            assert done and h == orc.hash(ref), d
            X, Y, Z = d
            assert (b.retire(t, (Y, Z, X)) == ref).all(), d
        ts = b.admit_many(grids, [s for _, s in worlds], n)
        b.run_segment()
        outs = [np.zeros_like(g) for g in grids]
        b.retire_many(ts, [o.ctypes.data for o in outs])
        for o, (d, seed), g in zip(outs, worlds, grids):
            ref = g.copy()
            orc.run(ref, seed, 0, n, nthreads=0)
            assert (o == ref).all(), d


def test_pipelined_steps_of_changing_sizes(fs3d, orc, cuda):
    """Seven pipelined steps, each admitting a different set of worlds (the
    staging buffers are reused round-robin and grow when a step needs more),
    with static materials in some worlds and pageable as well as page-locked
    inputs.  Every step's outputs equal the oracle."""
    S = 16
    rng = np.random.default_rng(7)
    steps = []
    for i in range(7):
        count = [3, 9, 2, 14, 5, 11, 4][i]
        worlds = small_batch(fs3d, 200 + i, count, max_dim=48 + 16 * (i % 3))
        grids = _with_statics(fs3d, worlds, every=2 + i % 2)
        pinned = i % 2 == 0
        if pinned:
            arena = cuda.from_numpy(np.concatenate([g.reshape(-1) for g in grids])).pin_memory()
            offs = np.concatenate([[0], np.cumsum([g.size for g in grids])[:-1]]).astype(np.int64)
            ptrs = [arena.data_ptr() + int(o) for o in offs]
            keep = arena
        else:
            keep = [g.copy() for g in grids]
            ptrs = [k.ctypes.data for k in keep]
        outs = [cuda.zeros(g.shape, dtype=cuda.uint8).pin_memory() for g in grids]
        start = int(rng.integers(0, 1000))
        steps.append((worlds, grids, ptrs, keep, outs, start))
    with fs3d.Batch(GiB, steps_per_segment=S) as b:
        prev = None
        for worlds, grids, ptrs, keep, outs, start in steps:
            ts = b.admit_many(None, [s for _, s in worlds], S, start_steps=[start] * len(worlds), ptrs=ptrs,
                              dims=[d for d, _ in worlds], wait=False)
            assert len(ts) == len(worlds)
            if prev is not None:
                b.retire_many(prev[0], [o.data_ptr() for o in prev[1]], wait=False)
            b.run_segment()
            prev = (ts, outs)
        b.retire_many(prev[0], [o.data_ptr() for o in prev[1]], wait=False)
        b.wait_copies()
        assert b.stats()["live_worlds"] == 0
    for worlds, grids, ptrs, keep, outs, start in steps:
        for (d, seed), g, o in zip(worlds, grids, outs):
            ref = g.copy()
            orc.run(ref, seed, start, S, nthreads=0)
            assert (o.numpy() == ref).all(), (d, start)


def test_retire_many_rejects_a_repeated_ticket(fs3d, orc):
    """A ticket listed twice in one retire_many is an argument error; nothing
    is retired and the batch stays usable."""
    worlds = small_batch(fs3d, 51, 3, max_dim=32)
    with fs3d.Batch(GiB, steps_per_segment=32) as b:
        ts = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, 32) for dims, seed in worlds]
        b.run_segment()
        with pytest.raises(fs3d.Fs3dError) as e:
            b.retire_many([ts[0], ts[1], ts[0]])
        assert e.value.status == fs3d.ERR_INVALID_ARG
        assert b.stats()["live_worlds"] == 3
        outs = [np.zeros((Y, Z, X), dtype=np.uint8) for (X, Y, Z), _ in worlds]
        b.retire_many(ts, [o.ctypes.data for o in outs])
        for o, (dims, seed) in zip(outs, worlds):
            assert (o == oracle_final(orc, fs3d, dims, seed, 32)).all()


def test_back_to_back_async_retires_into_scattered_pinned_outputs(fs3d, orc, cuda):
    """Four retire_many_async calls in a row, with no segment between them,
    into separately page-locked outputs (each its own allocation, so the
    device-side copy kernel writes them) of different world sizes.  Each
    call's copy jobs stay readable until its copy kernel has run, whatever the
    calls after it allocate; every output equals the oracle."""
    S = 24
    groups = [small_batch(fs3d, 300 + i, c, max_dim=m) for i, (c, m) in enumerate([(7, 96), (3, 32), (12, 64),
                                                                                   (5, 128)])]
    with fs3d.Batch(GiB, steps_per_segment=S) as b:
        tickets = []
        for worlds in groups:
            tickets.append([b.admit(fs3d.gen_batch_world(seed, *dims), seed, S) for dims, seed in worlds])
        b.run_segment()
        outs = []
        for worlds, ts in zip(groups, tickets):
            o = [cuda.zeros((Y, Z, X), dtype=cuda.uint8).pin_memory() for (X, Y, Z), _ in worlds]
            b.retire_many(ts, [t.data_ptr() for t in o], wait=False)
            outs.append(o)
        b.wait_copies()
        assert b.stats()["live_worlds"] == 0
    for worlds, o in zip(groups, outs):
        for (dims, seed), t in zip(worlds, o):
            assert (t.numpy() == oracle_final(orc, fs3d, dims, seed, S)).all(), dims


def test_read_many_snapshots_live_worlds(fs3d, orc, cuda):
    """read_many returns the worlds' state after the segments enqueued so far
    and leaves them running: the next segment continues from there."""
    S = 32
    worlds = small_batch(fs3d, 61, 9, max_dim=96)
    with fs3d.Batch(GiB, steps_per_segment=S) as b:
        ts = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, 3 * S) for dims, seed in worlds]
        b.run_segment()
        b.run_segment()
        snap = [cuda.zeros((Y, Z, X), dtype=cuda.uint8).pin_memory() for (X, Y, Z), _ in worlds]
        b.read_many(ts, [t.data_ptr() for t in snap])
        b.run_segment()  # must not touch the planes before the read-back has them
        assert b.stats()["live_worlds"] == len(worlds)
        outs = [np.zeros((Y, Z, X), dtype=np.uint8) for (X, Y, Z), _ in worlds]
        b.retire_many(ts, [o.ctypes.data for o in outs])
    for (dims, seed), sn, o in zip(worlds, snap, outs):
        assert (sn.numpy() == oracle_final(orc, fs3d, dims, seed, 2 * S)).all(), dims
        assert (o == oracle_final(orc, fs3d, dims, seed, 3 * S)).all(), dims


def test_poll_many_matches_single_polls_and_oracle(fs3d, orc):
    """poll_many reports the same done flags as one poll per world, and the
    hashes of the finished worlds (computed in one launch) equal the oracle's."""
    S = 32
    worlds = small_batch(fs3d, 71, 12, max_dim=96)
    steps = [10, 32, 40, 64, 70, 96, 5, 33, 64, 65, 20, 90]
    with fs3d.Batch(GiB, steps_per_segment=S) as b:
        ts = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, n) for (dims, seed), n in zip(worlds, steps)]
        b.run_segment()
        b.run_segment()
        b.sync()
        done, hs = b.poll_many(ts)
        for t, d, h, (dims, seed), n in zip(ts, done, hs, worlds, steps):
            assert bool(d) == (n <= 2 * S)
            if d:
                assert int(h) == orc.hash(oracle_final(orc, fs3d, dims, seed, n)), (dims, n)
                assert b.poll(t) == (1, int(h))
        b.retire_many([t for t, d in zip(ts, done) if d])
        b.run_segment()
        b.sync()
        rest = [t for t, d in zip(ts, done) if not d]
        done2, hs2 = b.poll_many(rest)
        assert done2.all()


def test_prepare_builds_tables_ahead_and_stays_exact(fs3d, orc):
    """fs3d_batch_prepare builds the next segment's tables while a segment is
    still running; an admission after it makes the segment build them again.
    Every world equals the oracle."""
    S = 16
    worlds = small_batch(fs3d, 81, 10, max_dim=64)
    steps = [S * 4, S * 3, S * 4, S * 2, 40, S * 4, 25, S * 4, S * 3, S * 4]
    with fs3d.Batch(GiB, steps_per_segment=S) as b:
        ts = [b.admit(fs3d.gen_batch_world(seed, *dims), seed, n) for (dims, seed), n in zip(worlds[:8], steps[:8])]
        b.prepare()
        b.run_segment()
        b.prepare()      # built while the first segment may still run
        b.run_segment()
        b.prepare()
        # an admission after the prepare: the next segment rebuilds its tables
        ts += [b.admit(fs3d.gen_batch_world(seed, *dims), seed, n) for (dims, seed), n in zip(worlds[8:], steps[8:])]
        for _ in range(4):
            b.run_segment()
            b.prepare()
        b.run_segment()
        b.sync()
        for t, (dims, seed), n in zip(ts, worlds, steps):
            done, h = b.poll(t)
            assert done
            assert h == orc.hash(oracle_final(orc, fs3d, dims, seed, n)), (dims, n)
