"""Serving loop over the batched entry points (no counterpart in the reference,
which extracts one volume per program run).

Requests for (resident volume, isovalue) pairs arrive over time.  Worker
slots -- each a context and a CUDA stream driven by its own host thread --
take every request that is waiting when they become free:

* Flying Edges requests with rows of at most 512 points run as one packed
  batch (iso_extract_batch_packed): counts, placement and meshes in one call,
  into the slot's reused buffers;
* the others, without a network, run one after another, one iso_extract_device
  call each into the context's reused single-request mesh (one count pass); with
  a network (predictor.Predictor), it sizes them from the resident volumes'
  block statistics and they run as one iso_extract_batch, a request whose mesh
  was too small going back to the head of the queue with the exact sizes the
  extraction reported (with `packed` off, the network or one iso_count_batch
  sizes every request of the batch).

A slot admits its work while it fits the device-memory budget beside the other
slots' (reused buffers count at their size); what does not fit waits.  Requests
that arrive while other slots work are taken by the next free slot, so the
slots' work overlaps on the device (continuous batching), but a slot starts
beside running work only behind a backlog.  While no slot is working and only a
few requests wait, the thread that receives them runs them itself, oldest
first, one extraction call each, with no hand-off to a slot.

`run_plain` is the loop to compare with: one request at a time, in arrival
order, iso_count_device, a mesh of exactly that size, iso_extract_device.
"""
import collections
import ctypes as C
import gc
import threading
import time

import numpy as np

from . import _lib
from .api import FLYING_EDGES, _algo, Batch, Context, DeviceMesh, PackedBuffers, Request, extract_batch_packed, make_grid
from ._lib import check, load


def mesh_bytes(n_points, n_tris, index_bytes=4):
    """Device bytes of a mesh: float3 points and normals, 3 indices per triangle."""
    return 24 * int(n_points) + 3 * index_bytes * int(n_tris)


def admit(sizes, in_use, budget, index_bytes=4):
    """How many of the waiting requests (their (n_points, n_tris) in arrival
    order) a slot admits: the longest prefix whose meshes fit beside `in_use`
    bytes under `budget`.  Returns (count, bytes).  A request larger than the
    whole budget is admitted alone once nothing else holds memory, so that it
    fails loudly instead of waiting forever."""
    total = 0
    count = 0
    for nv, nt in sizes:
        b = mesh_bytes(nv, nt, index_bytes)
        if in_use + total + b > budget:
            if count == 0 and in_use == 0:
                return 1, b
            break
        total += b
        count += 1
    return count, total


def carve_meshes(sizes, index_bytes, device):
    """Meshes of exactly the given (n_points, n_tris) as views into three
    allocations for the whole batch (not three per request).  Each mesh's
    triangles start on a 16-byte boundary (segments of a multiple of 4 rows)."""
    import torch
    nv = [max(int(v), 1) for v, _ in sizes]
    nt = [(max(int(t), 1) + 3) // 4 * 4 for _, t in sizes]
    pts = torch.empty((sum(nv), 3), dtype=torch.float32, device=device)
    nrm = torch.empty((sum(nv), 3), dtype=torch.float32, device=device)
    tri = torch.empty((sum(nt), 3), dtype=torch.int32 if index_bytes == 4 else torch.int64, device=device)
    out, ov, ot = [], 0, 0
    for (v, t), a, b in zip(sizes, nv, nt):
        m = DeviceMesh.__new__(DeviceMesh)
        m.index_bytes = index_bytes
        m.points, m.normals = pts[ov:ov + a], nrm[ov:ov + a]
        m.tris = tri[ot:ot + max(int(t), 1)]
        m.n_points = m.n_tris = 0
        out.append(m)
        ov += a
        ot += b
    return out


def poisson_arrivals(n, rate, seed=0):
    """n arrival times (seconds from the first) of a Poisson process of `rate` per second."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n)
    gaps[0] = 0.0
    return np.cumsum(gaps)


class Result:
    __slots__ = ("index", "arrival", "start", "done", "n_points", "n_tris", "mesh", "slot", "batch")

    def __init__(self, index, arrival):
        self.index = index
        self.arrival = arrival
        self.start = None  # when its first call was issued (seconds, the run's clock)
        self.done = None
        self.n_points = self.n_tris = 0
        self.mesh = None
        self.slot = -1
        self.batch = -1

    @property
    def latency(self):
        return self.done - self.arrival


def _request(volumes, vi, iso, algo):
    vol, dims = volumes[vi]
    return Request(vol, dims, iso, algo)


class Server:
    """Continuous batching over `slots` worker slots.

    volumes: list of (contiguous CUDA float32 tensor, dims) kept resident.
    budget_bytes: device memory the meshes in flight may hold.
    lanes: lanes of each slot's batches (0 leaves them to the autotuner).
    """

    def __init__(self, volumes, slots=2, max_batch=64, budget_bytes=120 << 30, lanes=8, device=0,
                 index_bytes=4, predictor=None):
        self.volumes = volumes
        self.slots = slots
        self.max_batch = max_batch
        self.budget = budget_bytes
        self.lanes = lanes
        self.device = device
        self.index_bytes = index_bytes
        self.contexts = [Context(device) for _ in range(slots)]
        self._singles = {}  # id(context) -> its single-request mesh
        # a slot's Flying Edges requests of rows up to 512 points run as one packed batch (iso_extract_batch_packed:
        # counts and meshes in one call, into the slot's buffers); the rest are sized by a count batch, or by the
        # network when there is one, and run as an extraction batch
        self.packed = True
        self._packed = {}  # id(context) -> its PackedBuffers
        self._streams = None
        # light load: while no slot is working and fewer than overlap_backlog requests wait, the thread that
        # receives them runs the oldest at once (no hand-off to a slot), with the plain calls on slot 0's
        # context (no slot runs meanwhile)
        self.inline_idle = True
        self.predictor = predictor
        # a slot that finds a single request waiting runs it with the plain calls (no count batch, no lanes)
        self.single_direct = True
        # a slot starts work beside other running work (a slot's batch or the receiving thread's request) only
        # once this many requests wait; fewer wait for the running work to end and then go together.  Two
        # single-request runs side by side take about 0.8-1.0 ms each against 0.36 ms alone (their kernels
        # share the L2 and their host round trips interleave), so at light load one thing runs at a time.
        self.overlap_backlog = 4
        # a slot takes the waiting requests as one batch once this many wait, else the oldest alone: at light
        # load a batch of two ends both at about 0.5 ms, one after the other they end at 0.28 and 0.57 ms
        self.batch_backlog = 1
        self.stats = None
        if predictor is not None:
            import torch
            from .predictor import block_stats
            self.stats = [block_stats(v, d) for v, d in volumes]
            torch.cuda.synchronize(device)  # the slots read them from their own streams
        for c in self.contexts:  # every batch differs: lanes launched directly, no graph capture
            check(load().iso_batch_set_lanes(c.handle, int(lanes)), c.handle)
            check(load().iso_batch_set_graph(c.handle, 0), c.handle)

    def _single_mesh(self, ctx, stream, n_points, n_tris):
        """The context's mesh for requests run alone: grown to at least (n_points, n_tris), a quarter more than
        asked, and kept for the next ones (the bytes count against the budget while they run)."""
        import torch
        m = self._singles.get(id(ctx))
        if m is None or m.points.shape[0] < n_points or m.tris.shape[0] < n_tris:
            cv = max(n_points, m.points.shape[0] if m is not None else 0)
            ct = max(n_tris, m.tris.shape[0] if m is not None else 0)
            self._singles[id(ctx)] = None
            with torch.cuda.stream(stream):
                m = DeviceMesh(cv + cv // 4 + 1024, ct + ct // 4 + 1024, self.index_bytes,
                               torch.device("cuda", self.device))
            self._singles[id(ctx)] = m
        return m

    @staticmethod
    def _packable(req):
        return _algo(req.algorithm) == FLYING_EDGES and req.dims[0] <= 512 and req.volume.data_ptr() % 16 == 0

    def _serve_packed(self, take, reqs, results, ctx, stream, state, cond, slot, t0, keep_meshes):
        """A slot's packed batch: one iso_extract_batch_packed into the slot's buffers (grown, and the batch
        run again, when it does not fit); the buffers count against the budget while it runs."""
        import torch

        bufs = self._packed.get(id(ctx))
        if bufs is None:
            with torch.cuda.stream(stream):
                bufs = PackedBuffers(0, 0, self.index_bytes, torch.device("cuda", self.device))
            self._packed[id(ctx)] = bufs
        with cond:
            while True:
                nbytes = mesh_bytes(bufs.points.shape[0], bufs.tris.shape[0], self.index_bytes)
                k, _ = admit([(bufs.points.shape[0], bufs.tris.shape[0])], state["in_use"], self.budget,
                             self.index_bytes)
                if k > 0 or state["error"]:
                    break
                state["admitting"] += 1
                cond.wait()
                state["admitting"] -= 1
            if k == 0:
                return
            state["in_use"] += nbytes
            batch_no = state["batches"]
            state["batches"] += 1
        try:
            with torch.cuda.stream(stream):
                meshes, _ = extract_batch_packed(reqs, buffers=bufs, index_bytes=self.index_bytes, ctx=ctx,
                                                 stream=stream.cuda_stream)
                grown = mesh_bytes(bufs.points.shape[0], bufs.tris.shape[0], self.index_bytes)
                if grown != nbytes:  # the buffers grew for this batch: count what they hold now
                    with cond:
                        state["in_use"] += grown - nbytes
                    nbytes = grown
                if keep_meshes:  # meshes of their own: the buffers serve the slot's next batch
                    kept = []
                    for m in meshes:
                        c = DeviceMesh(m.n_points, m.n_tris, self.index_bytes, torch.device("cuda", self.device))
                        c.points[: m.n_points].copy_(m.points[: m.n_points])
                        c.normals[: m.n_points].copy_(m.normals[: m.n_points])
                        c.tris[: m.n_tris].copy_(m.tris[: m.n_tris])
                        c.n_points, c.n_tris = m.n_points, m.n_tris
                        kept.append(c)
                    stream.synchronize()
                    meshes = kept
            done = time.perf_counter() - t0
            for i, m in zip(take, meshes):
                r = results[i]
                r.done = done
                r.n_points, r.n_tris = m.n_points, m.n_tris
                r.mesh = m if keep_meshes else None
                r.slot, r.batch = slot, batch_no
        finally:
            with cond:
                state["in_use"] -= nbytes
                if state["admitting"]:
                    cond.notify_all()

    def _serve_one(self, i, req, results, ctx, stream, state, cond, slot, t0, keep_meshes):
        """A request run alone (light load): one iso_extract_device into the context's single-request mesh,
        which holds every mesh seen so far (it grows, and the call runs again, when one does not fit)."""
        import torch

        lib = load()
        results[i].start = time.perf_counter() - t0
        sh = C.c_void_p(stream.cuda_stream)
        g = make_grid(req.dims, req.spacing, req.origin)
        a = req.descriptor().algorithm
        m = self._singles.get(id(ctx))
        if m is None:
            m = self._single_mesh(ctx, stream, 1, 1)
        nbytes = mesh_bytes(m.points.shape[0], m.tris.shape[0], self.index_bytes)
        with cond:
            while True:
                k, _ = admit([(m.points.shape[0], m.tris.shape[0])], state["in_use"], self.budget, self.index_bytes)
                if k > 0 or state["error"]:
                    break
                state["admitting"] += 1
                cond.wait()
                state["admitting"] -= 1
            if k == 0:
                return
            state["in_use"] += nbytes
            batch_no = state["batches"]
            state["batches"] += 1
        try:
            d = m.descriptor()
            st = lib.iso_extract_device(ctx.handle, a, req.volume.data_ptr(), C.byref(g), C.c_float(req.isoval),
                                        C.byref(d), sh)
            if st == _lib.ISO_ERR_CAPACITY:  # a mesh larger than any before: grow, run again
                m = self._single_mesh(ctx, stream, d.n_points, d.n_tris)
                grown = mesh_bytes(m.points.shape[0], m.tris.shape[0], self.index_bytes)
                with cond:
                    state["in_use"] += grown - nbytes
                nbytes = grown
                d = m.descriptor()
                st = lib.iso_extract_device(ctx.handle, a, req.volume.data_ptr(), C.byref(g),
                                            C.c_float(req.isoval), C.byref(d), sh)
            check(st, ctx.handle)
            kept = None
            if keep_meshes:  # a mesh of its own, the single-request mesh serves the next request
                with torch.cuda.stream(stream):
                    kept = DeviceMesh(d.n_points, d.n_tris, self.index_bytes, torch.device("cuda", self.device))
                    kept.points[: d.n_points].copy_(m.points[: d.n_points])
                    kept.normals[: d.n_points].copy_(m.normals[: d.n_points])
                    kept.tris[: d.n_tris].copy_(m.tris[: d.n_tris])
                stream.synchronize()
                kept.n_points, kept.n_tris = d.n_points, d.n_tris
            done = time.perf_counter() - t0
            r = results[i]
            r.done = done
            r.n_points, r.n_tris = d.n_points, d.n_tris
            r.mesh = kept
            r.slot, r.batch = slot, batch_no
        finally:
            with cond:
                state["in_use"] -= nbytes
                if state["admitting"]:  # memory for a request that waits for it
                    cond.notify_all()

    def run(self, requests, keep_meshes=False):
        """Serve `requests` = [(arrival seconds, volume index, isovalue, algorithm)] in real time.
        Returns one Result per request (latency = completion - arrival, seconds)."""
        lib = load()
        gc_was = gc.isenabled()
        gc.disable()  # no collector pauses in the middle of the stream
        try:
            return self._run(requests, keep_meshes, lib)
        finally:
            if gc_was:
                gc.enable()

    def _run(self, requests, keep_meshes, lib):
        import torch

        order = sorted(range(len(requests)), key=lambda i: requests[i][0])
        results = [None] * len(requests)
        queue = collections.deque()
        cond = threading.Condition()
        state = {"fed": False, "in_use": 0, "error": None, "batches": 0, "fallbacks": 0, "busy": 0, "admitting": 0}
        exact = {}  # request -> exact (n_points, n_tris) after a mesh came out too small
        t0 = time.perf_counter() + 0.002

        def wake():
            """(cond held) after work ended: wake the slots only if one may start (requests wait) or a request
            waits for memory -- needless wake-ups take the interpreter lock from the receiving thread"""
            if queue or state["admitting"]:
                cond.notify_all()

        if self._streams is None:  # one stream per slot for the server's life (the allocator caches per stream)
            self._streams = [torch.cuda.Stream(self.device) for _ in range(self.slots)]

        def worker(slot):
            ctx = self.contexts[slot]
            stream = self._streams[slot]
            try:
                while True:
                    with cond:
                        while not (state["error"] or (not queue and state["fed"]) or
                                   (queue and (state["busy"] == 0 or len(queue) >= self.overlap_backlog))):
                            cond.wait()
                        if state["error"] or (not queue and state["fed"]):
                            return
                        k = min(len(queue), self.max_batch) if len(queue) >= self.batch_backlog else 1
                        take = [queue.popleft() for _ in range(k)]
                        state["busy"] += 1
                    started = time.perf_counter() - t0
                    for i in take:
                        if results[i].start is None:
                            results[i].start = started
                    reqs = [_request(self.volumes, *requests[i][1:]) for i in take]
                    n = len(reqs)
                    if n == 1 and self.single_direct:
                        # one request waiting (light load): the plain calls on this slot's context -- an exact
                        # count and the extraction -- with none of the batch machinery around them
                        self._serve_one(take[0], reqs[0], results, ctx, stream, state, cond, slot, t0, keep_meshes)
                        with cond:
                            state["busy"] -= 1
                            wake()
                        continue
                    if self.packed:
                        pk = [q for q in range(n) if self._packable(reqs[q])]
                        if pk:
                            self._serve_packed([take[q] for q in pk], [reqs[q] for q in pk], results, ctx, stream,
                                               state, cond, slot, t0, keep_meshes)
                            rest = [q for q in range(n) if q not in set(pk)]
                            take = [take[q] for q in rest]
                            reqs = [reqs[q] for q in rest]
                            n = len(reqs)
                        if n and self.predictor is None and self.single_direct:
                            # the rest (rows longer than 512 points: large grids that fill the GPU alone) one
                            # after another, one extraction call each (one count pass, not a count batch and an
                            # extraction batch that count twice)
                            for i, req in zip(take, reqs):
                                self._serve_one(i, req, results, ctx, stream, state, cond, slot, t0, keep_meshes)
                            n = 0
                        if n == 0:
                            with cond:
                                state["busy"] -= 1
                                wake()
                            continue
                    if self.predictor is not None:
                        guess = [i for i in take if i not in exact]
                        caps = self.predictor.capacities(
                            [(self.stats[requests[i][1]], requests[i][2]) for i in guess], stream.cuda_stream)
                        pred = dict(zip(guess, caps))
                        sizes = [exact[i] if i in exact else pred[i] for i in take]
                    else:
                        arr = (_lib.IsoRequest * n)(*[r.descriptor() for r in reqs])
                        nv, nt = (C.c_int64 * n)(), (C.c_int64 * n)()
                        st = (C.c_int * n)()
                        check(lib.iso_count_batch(ctx.handle, n, arr, nv, nt, st, C.c_void_p(stream.cuda_stream)),
                              ctx.handle)
                        sizes = [(nv[i], nt[i]) for i in range(n)]
                    with cond:
                        while True:
                            k, nbytes = admit(sizes, state["in_use"], self.budget, self.index_bytes)
                            if k > 0 or state["error"]:
                                break
                            state["admitting"] += 1
                            cond.wait()  # another slot's meshes are holding the memory
                            state["admitting"] -= 1
                        if k == 0:
                            return
                        state["in_use"] += nbytes
                        for i in reversed(take[k:]):  # the rest goes back to the head of the queue
                            queue.appendleft(i)
                        batch_no = state["batches"]
                        state["batches"] += 1
                        if queue:  # the rest went back
                            cond.notify_all()
                    with torch.cuda.stream(stream):
                        meshes = carve_meshes(sizes[:k], self.index_bytes, torch.device("cuda", self.device))
                    codes = Batch(reqs[:k], meshes).run(ctx, stream.cuda_stream)
                    done = time.perf_counter() - t0
                    redo = [i for i, c in zip(take[:k], codes) if c == _lib.ISO_ERR_CAPACITY]
                    if any(c not in (0, _lib.ISO_ERR_CAPACITY) for c in codes) or (redo and self.predictor is None):
                        bad = [(i, requests[i][1:], sizes[q], (m.n_points, m.n_tris), c)
                               for q, (i, m, c) in enumerate(zip(take[:k], meshes, codes)) if c != 0]
                        raise RuntimeError("batch request failed (request, (volume, iso, algorithm), sized, "
                                           "reported, status): %s" % bad)
                    if redo:  # predicted too small: back to the head of the queue with the exact sizes
                        with cond:
                            for i, m, c in reversed(list(zip(take[:k], meshes, codes))):
                                if c == _lib.ISO_ERR_CAPACITY:
                                    exact[i] = (m.n_points, m.n_tris)
                                    queue.appendleft(i)
                            state["fallbacks"] += len(redo)
                            cond.notify_all()
                    for i, m, c in zip(take[:k], meshes, codes):
                        if c != 0:
                            continue
                        r = results[i]
                        r.done = done
                        r.n_points, r.n_tris = m.n_points, m.n_tris
                        r.mesh = m if keep_meshes else None
                        r.slot, r.batch = slot, batch_no
                    del meshes
                    with cond:
                        state["in_use"] -= nbytes
                        state["busy"] -= 1
                        wake()
            except BaseException as e:  # surfaced by run()
                with cond:
                    state["error"] = e
                    cond.notify_all()

        threads = [threading.Thread(target=worker, args=(s,), daemon=True) for s in range(self.slots)]
        for th in threads:
            th.start()
        # The receiving thread: arrived requests wait in `pending` (its own).  While no slot works and fewer
        # than overlap_backlog are pending, it runs the oldest itself with the plain calls, as the one-at-a-time
        # loop would, with no hand-off; otherwise it hands every pending request to the slots' queue.
        pending = collections.deque()
        pos = 0
        while pos < len(order) or pending:
            now = time.perf_counter() - t0
            while pos < len(order) and requests[order[pos]][0] <= now:
                q = order[pos]
                results[q] = Result(q, requests[q][0])
                pending.append(q)
                pos += 1
            if not pending:
                wait = t0 + requests[order[pos]][0] - time.perf_counter()
                if wait > 0:
                    time.sleep(wait)
                continue
            with cond:
                if state["error"]:
                    break
                inline = (self.inline_idle and not queue and state["busy"] == 0 and
                          len(pending) < self.overlap_backlog)
                if inline:
                    i = pending.popleft()
                    state["busy"] += 1  # the slots leave it alone
                else:
                    queue.extend(pending)
                    pending.clear()
                    cond.notify_all()
            if not inline:
                if pos < len(order):
                    wait = t0 + requests[order[pos]][0] - time.perf_counter()
                    if wait > 0:
                        time.sleep(wait)
                continue
            failed = None
            try:
                self._serve_one(i, _request(self.volumes, *requests[i][1:]), results, self.contexts[0],
                                torch.cuda.current_stream(self.device), state, cond, -1, t0, keep_meshes)
            except BaseException as e:  # surfaced after the slots have stopped
                failed = e
            with cond:
                state["busy"] -= 1
                if failed is not None:
                    state["error"] = failed
                    cond.notify_all()
                else:
                    wake()
            if failed is not None:
                break
        with cond:
            state["fed"] = True
            cond.notify_all()
        for th in threads:
            th.join()
        if state["error"]:
            raise state["error"]
        self.last_fallbacks = state["fallbacks"]
        return results


def run_plain(volumes, requests, device=0, index_bytes=4, keep_meshes=False):
    """One request at a time in arrival order: iso_count_device, allocate the
    mesh at that size, iso_extract_device.  Same Result records as Server.run."""
    import torch

    lib = load()
    ctx = Context(device)
    stream = torch.cuda.current_stream(device)
    sh = C.c_void_p(stream.cuda_stream)
    order = sorted(range(len(requests)), key=lambda i: requests[i][0])
    results = [None] * len(requests)
    gc_was = gc.isenabled()
    gc.disable()  # as the server: no collector pauses in the middle of the stream
    try:
        _plain_loop(lib, ctx, sh, volumes, requests, order, results, device, index_bytes, keep_meshes)
    finally:
        if gc_was:
            gc.enable()
    return results


def _plain_loop(lib, ctx, sh, volumes, requests, order, results, device, index_bytes, keep_meshes):
    import torch

    t0 = time.perf_counter() + 0.002
    for i in order:
        arrival, vi, iso, algo = requests[i]
        r = Result(i, arrival)
        results[i] = r
        wait = t0 + arrival - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        r.start = time.perf_counter() - t0
        req = _request(volumes, vi, iso, algo)
        g = make_grid(req.dims, req.spacing, req.origin)
        nv, nt = C.c_int64(), C.c_int64()
        a = req.descriptor().algorithm
        check(lib.iso_count_device(ctx.handle, a, req.volume.data_ptr(), C.byref(g), C.c_float(iso),
                                   C.byref(nv), C.byref(nt), sh), ctx.handle)
        m = DeviceMesh(nv.value, nt.value, index_bytes, torch.device("cuda", device))
        d = m.descriptor()
        check(lib.iso_extract_device(ctx.handle, a, req.volume.data_ptr(), C.byref(g), C.c_float(iso), C.byref(d),
                                     sh), ctx.handle)
        m.n_points, m.n_tris = d.n_points, d.n_tris
        r.done = time.perf_counter() - t0
        r.n_points, r.n_tris = m.n_points, m.n_tris
        r.mesh = m if keep_meshes else None
    return results


def summary(results, cells):
    """p50 / p99 latency (ms) and throughput of a run; cells[i] = cells of request i."""
    lat = np.array([r.latency for r in results]) * 1e3
    span = max(r.done for r in results) - min(r.arrival for r in results)
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "requests_per_s": len(results) / span,
            "Mcells_per_s": float(sum(cells)) / span / 1e6}
