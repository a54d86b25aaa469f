"""Batched FP32-refined Jacobi-PCG over many independent systems, with
continuous batching (no FEALPy counterpart: FEALPy's ``fealpy/solver/cg.py``
solves one system per call; this solves many at once on one GPU).

Every system keeps its own SELL-32 copy, FP64 solution and FP32 Krylov
vectors resident on the device.  The solver holds a fixed number of slots;
``add`` places a system into a free slot, ``step`` admits the pending systems,
runs the loop (one CUDA graph with a device-side while node) for at most a
given number of iterations, and retires every system that finished.  Systems
can be added between steps while others are in flight (continuous batching).

Each system's iterates depend only on that system: all its reductions run
over its own tiles in a fixed order, so a system solved alone and inside any
mix gives the same bits.
"""
import ctypes
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _lib
from . import kernels as K
from ._lib import call, ptr, stream_ptr
from .sparse import CSRTensor

__all__ = ["BatchSolver", "BatchResult", "solve_with_multigrid_lane"]


class BatchResult:
    """Outcome of one system: FP64 solution and its solve record."""

    def __init__(self, key, x, niter, relres, reason, n_updates):
        self.key, self.x, self.niter, self.relres, self.reason, self.n_updates = key, x, niter, relres, reason, n_updates
        self.fp64_iterations = 0  # of niter, those run in FP64 after an FP32 stagnation

    def info(self):
        return {"niter": self.niter, "relres": self.relres, "reason": self.reason, "n_updates": self.n_updates}


class _Slot:
    def __init__(self, key, S, dinv64, b, x, vecs, rtol, maxit, fp64, A):
        self.key, self.S, self.dinv64, self.b, self.x, self.vecs = key, S, dinv64, b, x, vecs
        self.rtol, self.maxit, self.fp64, self.A = rtol, maxit, fp64, A
        self.admitted = False
        self.iters_before = 0  # FP32 iterations spent before an FP64 continuation
        self.tiles = None      # cached (slice tile bounds, row tile bounds)


class BatchSolver:
    """Continuous-batching mixed-precision PCG.

    ``slices_per_tile`` / ``rows_per_tile`` / ``slice_threads`` set the work
    split of the batched kernels (see :func:`autotune`)."""

    def __init__(self, max_systems: int = 256, *, max_slice_tiles: int = 1 << 16, max_row_tiles: int = 1 << 16,
                 slices_per_tile: int = 8, rows_per_tile: int = 1024, slice_threads: int = 256,
                 max_tiles_per_system: int = 16384, delta: float = 0.1, device=None):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.max_systems = int(max_systems)
        self.max_slice_tiles, self.max_row_tiles = int(max_slice_tiles), int(max_row_tiles)
        self.slices_per_tile, self.rows_per_tile = int(slices_per_tile), int(rows_per_tile)
        self.slice_threads = int(slice_threads)
        self.max_tiles_per_system = int(max_tiles_per_system)
        self.delta = float(delta)
        lib = _lib.lib()
        nbytes = int(lib.fgb_batch_bytes(self.max_systems, self.max_slice_tiles, self.max_row_tiles))
        if nbytes == 0:
            raise ValueError("invalid batch capacities")
        self._buf = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        h = ctypes.c_void_p()
        call("fgb_batch_create", self.max_systems, self.max_slice_tiles, self.max_row_tiles, self.slice_threads,
             ptr(self._buf), nbytes, ctypes.byref(h))
        self._h = h
        self._slots: List[Optional[_Slot]] = [None] * self.max_systems
        self._dirty = True
        self._n_table = 0
        self.launches = 0
        self.used_graph = False
        self.fallbacks = 0  # systems continued in FP64 after their FP32 iterations stagnated

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().fgb_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    # ------------------------------------------------------------ systems
    def free_slots(self) -> int:
        return sum(1 for s in self._slots if s is None)

    def active(self) -> int:
        return self.max_systems - self.free_slots()

    def _n_tiles(self, lim, per_tile):
        step = max(per_tile, -(-lim // self.max_tiles_per_system))
        return -(-lim // step)

    def fits(self, n: int) -> bool:
        """Whether a free slot and the tile tables have room for one more
        system of ``n`` rows next to the systems already placed."""
        if self.free_slots() == 0:
            return False
        st = vt = 0
        for sl in self._slots:
            if sl is not None:
                st += self._n_tiles(sl.S.n_slices, self.slices_per_tile)
                vt += self._n_tiles(sl.S.n, self.rows_per_tile)
        st += self._n_tiles(int(_lib.lib().fgb_sell_slots(n)) // 32, self.slices_per_tile)
        vt += self._n_tiles(n, self.rows_per_tile)
        return st <= self.max_slice_tiles and vt <= self.max_row_tiles

    @staticmethod
    def resident_bytes(n: int, nnz_padded: int, fp64_values: bool) -> int:
        """Device bytes one system keeps resident (SELL copy + vectors)."""
        return nnz_padded * (4 + 4 + (8 if fp64_values else 0)) + n * (8 + 8 + 8 + 6 * 4) + (n // 32 + 2) * 12

    def add(self, A: CSRTensor, b: torch.Tensor, x0: Optional[torch.Tensor] = None, *, rtol: float = 1e-10,
            maxit: int = 100000, key=None, fp64: bool = False) -> int:
        """Place ``A x = b`` in a free slot (admitted at the next ``step``);
        returns the slot.  An FP32 ``A`` is its own operator; an FP64 ``A``
        keeps FP64 values for the residual recomputation.  ``fp64``: iterate
        in FP64 (plain FP64 PCG with the same stopping rule).  An FP32 system
        that stagnates is continued in FP64 from its current iterate."""
        if not isinstance(A, CSRTensor):
            raise NotImplementedError("BatchSolver takes CSRTensor matrices")
        try:
            slot = self._slots.index(None)
        except ValueError:
            raise RuntimeError("no free slot in the batch") from None
        n = A.shape[0]
        if fp64:
            S = K.sell_build(A.crow, A.col, A.values.to(torch.float64).contiguous(), None, want64=True, want32=False,
                             d16=False)
        elif A.values.dtype == torch.float32:
            S = K.sell_build(A.crow, A.col, None, A.values.contiguous(), want64=False, want32=True, d16=False)
        else:
            S = K.sell_build(A.crow, A.col, A.values.to(torch.float64).contiguous(), None, want64=True, want32=True,
                             d16=False)
        dinv64 = A.diagonal_inverse().to(torch.float64).contiguous()
        b64 = b.to(self.device, torch.float64).contiguous()
        x = torch.zeros(n, dtype=torch.float64, device=self.device) if x0 is None else \
            x0.to(self.device, torch.float64).clone()
        vecs = torch.empty((6, n), dtype=torch.float64 if fp64 else torch.float32, device=self.device)
        self._slots[slot] = _Slot(slot if key is None else key, S, dinv64, b64, x, vecs, float(rtol), int(maxit),
                                  bool(fp64), A)
        self._dirty = True
        return slot

    # ------------------------------------------------------------ tables
    def _tile_bounds(self, lim, per_tile):
        """(begin, end) of one system's tiles: ``per_tile`` slices (rows),
        widened so that the system has at most ``max_tiles_per_system`` tiles
        (its per-system sums stay short).  Depends on the system only."""
        step = max(per_tile, -(-lim // self.max_tiles_per_system))
        b = np.arange(0, lim, step, dtype=np.int32)
        return np.stack([b, np.minimum(b + step, lim).astype(np.int32)], axis=1)

    def _tiles(self, parts):
        """Tile array (sys, begin, end, 0) int32 and tile pointers of the
        table from each slot's cached bounds (None for an empty slot)."""
        rows, ptr_ = [], [0]
        for s, bnd in enumerate(parts):
            if bnd is not None and len(bnd):
                t = np.zeros((len(bnd), 4), dtype=np.int32)
                t[:, 0] = s
                t[:, 1:3] = bnd
                rows.append(t)
            ptr_.append(ptr_[-1] + (0 if bnd is None else len(bnd)))
        tiles = np.ascontiguousarray(np.concatenate(rows) if rows else np.zeros((1, 4), dtype=np.int32))
        return tiles, np.asarray(ptr_, dtype=np.int32), ptr_[-1]

    def _sync_tables(self):
        used = [i for i, s in enumerate(self._slots) if s is not None]
        n_sys = (max(used) + 1) if used else 0
        systems = (_lib.BatchSystem * max(n_sys, 1))()
        slice_parts, row_parts = [], []
        for i in range(n_sys):
            sl = self._slots[i]
            if sl is None:
                slice_parts.append(None)
                row_parts.append(None)
                continue
            S, v = sl.S, sl.vecs
            d = systems[i]
            d.n, d.n_slices = S.n, S.n_slices
            d.slice_ptr, d.perm, d.col = S.slice_ptr.data_ptr(), S.perm.data_ptr(), S.col.data_ptr()
            d.val32 = S.val32.data_ptr() if S.val32 is not None else None
            d.val64 = S.val64.data_ptr() if S.val64 is not None else None
            d.fp64 = 1 if sl.fp64 else 0
            d.dinv64, d.b, d.x = sl.dinv64.data_ptr(), sl.b.data_ptr(), sl.x.data_ptr()
            d.r, d.z, d.p, d.Ap, d.y, d.dinv32 = (v[k].data_ptr() for k in range(6))
            if sl.tiles is None:
                sl.tiles = (self._tile_bounds(S.n_slices, self.slices_per_tile),
                            self._tile_bounds(S.n, self.rows_per_tile))
            slice_parts.append(sl.tiles[0])
            row_parts.append(sl.tiles[1])
        sta, spa, nst = self._tiles(slice_parts)
        vta, vpa, nvt = self._tiles(row_parts)
        if nst > self.max_slice_tiles or nvt > self.max_row_tiles:
            raise RuntimeError("batch tile capacity exceeded: raise max_slice_tiles / max_row_tiles")
        vp_ = ctypes.c_void_p
        call("fgb_batch_set", self._h, n_sys, systems, nst, vp_(sta.ctypes.data), vp_(spa.ctypes.data), nvt,
             vp_(vta.ctypes.data), vp_(vpa.ctypes.data), stream_ptr(self.device))
        self._n_table = n_sys
        self._dirty = False

    # ------------------------------------------------------------ running
    def step(self, max_iterations: int = 1 << 40, graph: bool = True) -> List[BatchResult]:
        """Admit pending systems, iterate all unfinished ones for at most
        ``max_iterations`` iterations, retire and return those that finished."""
        stream = stream_ptr(self.device)
        pending = [i for i, s in enumerate(self._slots) if s is not None and not s.admitted]
        if self._dirty:
            self._sync_tables()
        if pending:
            n = len(pending)
            slots = (ctypes.c_int32 * n)(*pending)
            rt = (ctypes.c_double * n)(*[self._slots[i].rtol for i in pending])
            mx = (ctypes.c_int64 * n)(*[self._slots[i].maxit for i in pending])
            call("fgb_batch_admit", self._h, n, slots, rt, mx, self.delta, stream)
            self.launches += 5
            for i in pending:
                self._slots[i].admitted = True
        if self._n_table == 0:
            return []
        states = (_lib.BatchState * self._n_table)()
        running = ctypes.c_int32()
        graphed = ctypes.c_int32()
        call("fgb_batch_run", self._h, int(max_iterations), int(bool(graph)), states, ctypes.byref(running),
             ctypes.byref(graphed), stream)
        self.used_graph = bool(graphed.value)
        done = [i for i in range(self._n_table) if self._slots[i] is not None and states[i].done != 0]
        out = []
        if done:
            arr = (ctypes.c_int32 * len(done))(*done)
            call("fgb_batch_retire", self._h, len(done), arr, stream)
            restart = []
            for i in done:
                sl, stt = self._slots[i], states[i]
                self._slots[i] = None
                if stt.done == 7 and not sl.fp64:  # FP32 iterations stagnated: continue in FP64 from x
                    restart.append((sl, int(stt.niter), int(stt.n_updates)))
                    continue
                if stt.done == 4:  # zero right-hand side: x = 0
                    sl.x.zero_()
                res = BatchResult(sl.key, sl.x, sl.iters_before + int(stt.niter), float(stt.true_rel),
                                  int(stt.done), int(stt.n_updates))
                res.fp64_iterations = int(stt.niter) if sl.fp64 and sl.iters_before else 0
                out.append(res)
            for sl, it, nu in restart:
                self.fallbacks += 1
                slot = self.add(sl.A, sl.b, sl.x, rtol=sl.rtol, maxit=max(sl.maxit - it, 1), key=sl.key, fp64=True)
                self._slots[slot].iters_before = sl.iters_before + it
            self._dirty = True
        return out

    def solve_all(self, graph: bool = True) -> Dict[object, BatchResult]:
        """Run until every system in the batch has finished."""
        res = {}
        while self.active():
            for r in self.step(graph=graph):
                res[r.key] = r
        return res

    # ------------------------------------------------------------ tuning
    def spmv_time_us(self, reps: int = 10) -> float:
        """Mean time of one batched FP32 SpMV over every system in the table."""
        if self._dirty:
            self._sync_tables()
        n = self._n_table
        xs = (ctypes.c_void_p * max(n, 1))()
        ys = (ctypes.c_void_p * max(n, 1))()
        keep = []
        for i in range(n):
            sl = self._slots[i]
            if sl is None:
                continue
            x = torch.ones(sl.S.n, dtype=torch.float32, device=self.device)
            y = torch.empty_like(x)
            keep += [x, y]
            xs[i], ys[i] = x.data_ptr(), y.data_ptr()
        stream = stream_ptr(self.device)
        s = torch.cuda.current_stream(self.device)
        call("fgb_batch_spmv", self._h, xs, ys, stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            call("fgb_batch_spmv", self._h, xs, ys, stream)
        e1.record(s)
        e1.synchronize()
        return 1000.0 * e0.elapsed_time(e1) / reps


def autotune(systems, candidates=((4, 256), (8, 256), (16, 256), (8, 512), (16, 512), (8, 1024)),
             device=None, **kw) -> Dict[tuple, float]:
    """Choose (slices per tile, threads per block) of the batched slice
    kernels by timing the batched SpMV of ``systems`` (a list of (A, b)) for
    each candidate; returns {candidate: microseconds}."""
    times = {}
    for spt, thr in candidates:
        bs = BatchSolver(max(len(systems), 1), slices_per_tile=spt, slice_threads=thr, device=device, **kw)
        for A, b in systems:
            bs.add(A, b)
        times[(spt, thr)] = bs.spmv_time_us()
        del bs
    return times


def solve_with_multigrid_lane(batch: BatchSolver, lane_systems, *, workers: int = 4, fp64: bool = False,
                              graph: bool = True) -> Dict[object, BatchResult]:
    """Solve the systems already added to ``batch`` and, at the same time, the
    ``lane_systems`` ([(key, A, b, rtol, maxit)]) by multigrid PCG
    (:func:`fealpy_gb300.amg.multigrid_solve`) on ``workers`` threads, each
    with its own CUDA stream.  Large systems, whose Jacobi iterations would
    set the batch's makespan, go to the lane.  Returns every result by key
    (lane results: ``reason`` from PCG, ``n_updates`` 0).  Call with the
    current stream idle of other work on the lane systems' data."""
    import threading
    from concurrent.futures import ThreadPoolExecutor
    from .amg import multigrid_solve
    local = threading.local()
    ready = torch.cuda.Event()
    ready.record(torch.cuda.current_stream(batch.device))

    def job(key, A, b, rtol, maxit):
        st = getattr(local, "stream", None)
        if st is None:
            st = local.stream = torch.cuda.Stream(batch.device)
        with torch.cuda.stream(st):
            st.wait_event(ready)
            x, niter, reason, relres = multigrid_solve(A, b, rtol, maxit, fp64)
            st.synchronize()
        return BatchResult(key, x, niter, relres, reason, 0)

    with ThreadPoolExecutor(max(int(workers), 1)) as pool:
        futs = [pool.submit(job, *s) for s in lane_systems]
        out = batch.solve_all(graph=graph) if batch.active() else {}
        for f in futs:
            r = f.result()
            out[r.key] = r
    return out
