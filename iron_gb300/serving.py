"""Serving loop: a persistent engine for a stream of assembly + solve requests.

Requests are Laplace/diffusion problems (trilinear hexahedra, per-element conductivity, u = 0 at
x = 0 and u = 1 at x = 1, solved to a relative residual of 1e-10) or Mooney-Rivlin problems
(triquadratic u / trilinear p, per-request c10 and c01 and stretch lambda: one uniaxial load step
solved by Newton's method from the affine predictor to Iron's default tolerances -- absolute
1e-10 and relative 1e-5 on the residual norm, 1e-5 on the step, linear solves to 1e-5 --
with the consistent tangent and a cubic backtracking line search) on jittered regular meshes of
different sizes.  The engine

* admits requests in arrival order as soon as a worker slot is free and the request's device
  memory fits the HBM budget (a request that does not fit yet may be overtaken by later ones that
  do; least-recently-used resident state that no running request holds is evicted to make room);
* keeps per-size state resident: mesh connectivity, colouring, the Iron-identical CSR structure,
  the MR slot map, and per-worker value/vector buffers;
* runs each worker on its own CUDA stream, so requests admitted while others are on the GPU
  overlap with them (continuous batching);
* replays CUDA graphs for the launch-bound Laplace requests: per (worker, mesh size) one graph for
  "assemble + CG start" and one for "25 CG iterations + status copy", replayed until the device
  says the solve has converged;
* batches small Laplace requests: up to LAPLACE_BATCH queued requests of the same side
  (side <= BATCH_MAX_N) run together through one pair of graphs holding every request's launch
  sequence, so a single graph launch advances all of them and one status check per chunk serves
  the batch.  Each request's sequence is its single-request sequence on its own buffers, so its
  result is the one it has alone.
  Mooney-Rivlin requests (milliseconds-long kernels and host-side Newton control) run eagerly
  on their worker's stream.

Kernels are deterministic (coloured scatters, fixed-order reductions), so a request's result does
not depend on what runs beside it.  `plain_fp64` is the baseline: the FP64 drop-in path run one
request at a time, building each request's structure from scratch as Iron does per problem.
"""
from __future__ import annotations

import copy
import ctypes as C
import math
import threading
import time
from collections import OrderedDict, deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._lib import GfeError
from .elasticity import MooneyRivlinAssembly
from .laplace import LaplaceAssembly
from .mesh import RegularMesh, linear_component
from .newton import NewtonSolver, uniaxial_roller_conditions

LAPLACE_RTOL = 1e-10
MR_STRETCH = (1.0, 1.1)
CG_CHUNK = 25
# small Laplace requests of one side are served in batches of up to LAPLACE_BATCH
LAPLACE_BATCH = 8
BATCH_MAX_N = 16
# share of the device torch's caching allocator may hold while an engine runs (the rest stays
# free for the library's stream-ordered scratch)
TORCH_MEMORY_FRACTION = 0.85
# times a request that ran out of device memory is retried (after the engine has drained and
# released the allocator's cache)
OOM_RETRIES = 2


# engines alive in the process: the allocator cap is lifted when the last one closes
_ENGINES = {"live": 0}
_ENGINES_LOCK = threading.Lock()


def _is_out_of_memory(e: BaseException) -> bool:
    return isinstance(e, torch.cuda.OutOfMemoryError) or (isinstance(e, GfeError) and e.status == -7)


# torch registers every captured graph with the process-wide CUDA generator state, which is not
# safe against concurrent capture or destruction from several threads.  Capture, destruction and
# the building of resident state all happen under this lock, taken before the engine's own lock
# whenever both are held.
_GRAPH_LOCK = threading.RLock()


class _CgState(C.Structure):
    _fields_ = [("rr", C.c_double), ("rr0", C.c_double), ("done", C.c_int32), ("iterations", C.c_int32),
                ("breakdown", C.c_int32), ("reserved", C.c_int32)]


# ---- requests -----------------------------------------------------------------------------------

@dataclass
class Request:
    rid: int
    kind: str  # "laplace" | "mr"
    n: int
    seed: int
    arrival: float = 0.0
    # client-side inputs (host, pinned once generated)
    inputs: dict = field(default_factory=dict, repr=False)
    # filled by the engine
    t_admit: float = math.nan
    t_done: float = math.nan
    result: np.ndarray | None = field(default=None, repr=False)
    info: dict = field(default_factory=dict)
    cancelled: bool = False

    def cancel(self) -> None:
        """Withdraw the request.  A request still queued (not yet admitted) is dropped by the
        engine and never runs; one already admitted runs to completion."""
        self.cancelled = True

    @property
    def elements(self) -> int:
        return self.n ** 3

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


def request_stream(n_requests: int = 2000, rate: float = 200.0, laplace_fraction: float = 0.7, n_lo: int = 4,
                   n_hi: int = 64, seed: int = 0, mr_n_hi: int | None = None) -> list[Request]:
    """Poisson arrivals (exponential inter-arrival times at `rate` per second), kind Laplace with
    probability laplace_fraction else Mooney-Rivlin, side n = round(exp(U(ln n_lo, ln n_hi))).
    mr_n_hi: a smaller upper side for the Mooney-Rivlin requests (the same uniform draw, mapped
    onto [ln n_lo, ln mr_n_hi]); None keeps n_hi."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    kinds = np.where(rng.random(n_requests) < laplace_fraction, "laplace", "mr")
    u = rng.uniform(0.0, 1.0, n_requests)
    hi = np.where(kinds == "mr", mr_n_hi if mr_n_hi is not None else n_hi, n_hi).astype(float)
    ns = np.rint(np.exp(math.log(n_lo) + u * (np.log(hi) - math.log(n_lo)))).astype(int)
    seeds = rng.integers(0, 2 ** 31 - 1, n_requests)
    return [Request(i, str(kinds[i]), int(ns[i]), int(seeds[i]), float(t[i] - t[0])) for i in range(n_requests)]


def _pinned(a: np.ndarray) -> torch.Tensor:
    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.pin_memory() if torch.cuda.is_available() else t


def make_inputs(req: Request, pin: bool = True) -> None:
    """The client's data for a request (host memory): jittered coordinates and conductivity
    (Laplace) or coordinates, material and stretch (Mooney-Rivlin)."""
    rng = np.random.default_rng(req.seed)
    conv = _pinned if pin else (lambda a: torch.from_numpy(np.ascontiguousarray(a)))
    if req.kind == "laplace":
        m = RegularMesh((req.n,) * 3)
        m.jitter_interior(int(rng.integers(2 ** 31)))
        kappa = np.exp(rng.uniform(math.log(0.1), math.log(10.0), m.n_elements))
        req.inputs = {"coords": conv(m.coords), "kappa": conv(kappa)}
    else:
        m = RegularMesh((req.n,) * 3, order=2)
        m.jitter_interior(int(rng.integers(2 ** 31)))
        c = np.exp(rng.uniform(math.log(0.5), math.log(10.0), 2))
        lam = rng.uniform(*MR_STRETCH)
        req.inputs = {"coords": conv(m.coords), "c": conv(c), "lam": float(lam)}


def _laplace_bcs(m: RegularMesh):
    fixed = np.zeros(m.n_nodes, np.uint8)
    x0 = np.zeros(m.n_nodes)
    fixed[m.face_nodes(0, 0)] = 1
    right = m.face_nodes(0, 1)
    fixed[right] = 1
    x0[right] = 1.0
    return fixed, x0


# ---- resident state --------------------------------------------------------------------------------

class _LaplaceMesh:
    """Per-size resident Laplace state: connectivity, colouring, CSR structure, BCs."""

    def __init__(self, n: int, dev):
        m = RegularMesh((n, n, n))
        self.mesh = m
        base = LaplaceAssembly.from_regular_mesh(m, device=dev)
        if base.regular is None:
            raise GfeError(-3, "generated mesh failed the regular-structure check")
        self.base = base
        fixed, x0 = _laplace_bcs(m)
        self.fixed = torch.from_numpy(fixed).to(dev)
        self.x0 = torch.from_numpy(x0).to(dev)
        base.values = None  # the base object holds structure only


def laplace_batch_capacity(n: int) -> int:
    """Requests one Laplace slot of side n serves at once."""
    return LAPLACE_BATCH if n <= BATCH_MAX_N else 1


class _LaplaceEntry:
    """One request's buffers in a Laplace slot, and its two launch sequences (which the slot's
    graphs capture)."""

    def __init__(self, lm: _LaplaceMesh, dev):
        b = lm.base
        self.lm = lm
        self.asm = copy.copy(b)
        self.asm.__dict__.pop("_ws_cache", None)  # a worker's assembly workspaces are its own
        # valid data for the warm-up run before capture: the undeformed mesh, unit conductivity
        self.asm.coords = b.coords.clone()
        self.asm.kappa = torch.ones(b.n_elements, dtype=torch.float64, device=dev)
        self.asm.values = torch.empty(b.nnz, dtype=torch.float64, device=dev)
        self.asm.values32 = torch.empty(b.nnz, dtype=torch.float32, device=dev)
        self.asm.rhs = torch.empty(b.n_nodes, dtype=torch.float64, device=dev)
        self.x = torch.empty(b.n_nodes, dtype=torch.float64, device=dev)
        L = _lib.load()
        wsb = int(L.gfe_cg_workspace_bytes(b.n_nodes))
        self.ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        nx, ny, nz = b.regular
        awb = int(L.gfe_laplace_regular_workspace_bytes(nx, ny, nz, 2))
        self.asm_ws = torch.empty(max(awb, 16), dtype=torch.uint8, device=dev)
        self.state = torch.zeros(C.sizeof(_CgState), dtype=torch.uint8).pin_memory()

    def begin(self, stream):
        a = self.asm
        nx, ny, nz = a.regular
        st = _lib.stream_handle(stream)
        self.x.copy_(self.lm.x0)
        _lib.call("gfe_laplace_assemble_regular_ws", nx, ny, nz, _lib.ptr(a.coords), _lib.ptr(a.kappa),
                  _lib.ptr(a.row_ptr), _lib.ptr(a.values), _lib.ptr(a.values32), _lib.ptr(a.rhs), 2,
                  _lib.ptr(self.asm_ws), st)
        _lib.call("gfe_cg_begin", a.n_nodes, _lib.ptr(a.row_ptr), _lib.ptr(a.col_idx), _lib.ptr(a.values), None,
                  _lib.ptr(self.lm.fixed), _lib.ptr(self.x), LAPLACE_RTOL, _lib.ptr(self.ws), st)

    def chunk(self, stream):
        a = self.asm
        st = _lib.stream_handle(stream)
        _lib.call("gfe_cg_steps", a.n_nodes, _lib.ptr(a.row_ptr), _lib.ptr(a.col_idx), _lib.ptr(a.values),
                  _lib.ptr(self.lm.fixed), _lib.ptr(self.x), CG_CHUNK, _lib.ptr(self.ws), st)
        _lib.call("gfe_cg_status", a.n_nodes, _lib.ptr(self.ws), C.c_void_p(self.state.data_ptr()), st)

    def load(self, req: Request) -> None:
        """Queue the copies of a request's inputs (pinned host memory) on the current stream."""
        self.asm.coords.copy_(req.inputs["coords"], non_blocking=True)
        self.asm.kappa.copy_(req.inputs["kappa"], non_blocking=True)


class _LaplaceSlot:
    """A worker's buffers and captured graphs for one Laplace mesh size: laplace_batch_capacity(n)
    entries.  A batch of k requests runs on the first w entries, w the width of the batch (the
    next power of two, at most the capacity); entries past k repeat the last request's inputs and
    their results are dropped.  All entries run on the worker's stream, one after the other, so a
    graph is captured from that one stream only."""

    def __init__(self, lm: _LaplaceMesh, dev, use_graphs: bool):
        self.lm = lm
        cap = laplace_batch_capacity(lm.mesh.nelem[0])
        self.entries = [_LaplaceEntry(lm, dev) for _ in range(cap)]
        self.use_graphs = use_graphs
        self.graphs: dict = {}  # width -> (begin graph, chunk graph)
        self.warm: set = set()

    @property
    def capacity(self) -> int:
        return len(self.entries)

    def width(self, k: int) -> int:
        w = 1
        while w < k:
            w *= 2
        return min(w, self.capacity)

    def _fork(self, stream, w: int, step: str) -> None:
        """Queue entries[0:w]'s `step` ("begin" | "chunk") on `stream`."""
        for e in self.entries[:w]:
            getattr(e, step)(stream)

    def capture(self, stream, w: int = 1):
        """Warm up the width-w launch sequences once eagerly, then (with graphs on) capture both
        on `stream`.  Capture is thread-local (other workers keep launching and allocating
        meanwhile) and, unlike torch.cuda.graph, does not synchronise the whole device first."""
        with torch.cuda.stream(stream):
            if w not in self.warm:
                self._fork(stream, w, "begin")
                self._fork(stream, w, "chunk")
                stream.synchronize()
                self.warm.add(w)
            if not self.use_graphs:
                return
            graphs = []
            with _GRAPH_LOCK:
                for step in ("begin", "chunk"):
                    g = torch.cuda.CUDAGraph()
                    g.capture_begin(capture_error_mode="thread_local")
                    try:
                        self._fork(stream, w, step)
                    finally:
                        g.capture_end()
                    graphs.append(g)
            self.graphs[w] = tuple(graphs)
        stream.synchronize()

    def release(self):
        with _GRAPH_LOCK:
            self.graphs = {}

    @property
    def n_graphs(self) -> int:
        return 2 * len(self.graphs)

    def run(self, reqs: list[Request], stream) -> None:
        """Solve `reqs` (1 to capacity requests of this slot's side) together."""
        if not 1 <= len(reqs) <= self.capacity:
            raise GfeError(-1, f"a Laplace slot of capacity {self.capacity} got {len(reqs)} requests")
        w = self.width(len(reqs))
        if w not in (self.graphs if self.use_graphs else self.warm):
            with _GRAPH_LOCK:
                self.capture(stream, w)
        with torch.cuda.stream(stream):
            for i, e in enumerate(self.entries[:w]):
                e.load(reqs[min(i, len(reqs) - 1)])
            if self.use_graphs:
                self.graphs[w][0].replay()
            else:
                self._fork(stream, w, "begin")
            states = [_CgState.from_address(e.state.data_ptr()) for e in self.entries[:w]]
            chunks = 0
            while True:
                if self.use_graphs:
                    self.graphs[w][1].replay()
                else:
                    self._fork(stream, w, "chunk")
                chunks += 1
                stream.synchronize()
                if all(st.done for st in states) or chunks * CG_CHUNK > 200000:
                    break
            outs = []
            for e in self.entries[: len(reqs)]:
                out = torch.empty(e.x.numel(), dtype=torch.float64, pin_memory=True)
                out.copy_(e.x, non_blocking=True)
                outs.append(out)
            stream.synchronize()
        bits = _lib.device_errors(stream)
        for req, st, out in zip(reqs, states, outs):
            if bits or st.done != 2:
                raise GfeError(-5, f"request {req.rid}: Laplace solve ended with state {st.done}, "
                                   f"device bits {bits:#x}")
            req.result = out.numpy()
            req.info = {"iterations": int(st.iterations), "rel_residual": math.sqrt(st.rr / st.rr0) if st.rr0 else 0.0,
                        "batch": len(reqs)}


class _MRMesh:
    """Per-size resident Mooney-Rivlin state: connectivity, colouring, CSR structure, slot map."""

    def __init__(self, n: int, dev):
        self.base = MooneyRivlinAssembly.from_regular_mesh((n, n, n), device=dev)
        b = self.base
        b.values = None
        # the Dirichlet DOFs (rollers and the pulled face): boundary nodes are never jittered, so
        # the mask holds for every request of this size
        self.fixed, _ = uniaxial_roller_conditions(b, 1.0)


class _MRSlot:
    """One Mooney-Rivlin request's working state: its coordinates, values and solution."""

    def __init__(self, mm: _MRMesh, dev):
        b = mm.base
        self.mm = mm
        self.asm = copy.copy(b)
        self.asm.__dict__.pop("_ws_cache", None)  # a worker's assembly workspaces are its own
        self.asm.xg = torch.empty_like(b.xg)
        self.asm.values = torch.empty(b.nnz, dtype=torch.float64, device=dev)
        self.dep = torch.empty(b.ndof, dtype=torch.float64, device=dev)

    def run(self, req: Request, stream, precision: str = "mixed") -> None:
        a = self.asm
        with torch.cuda.stream(stream):
            a.xg.copy_(req.inputs["coords"], non_blocking=True)
            c = req.inputs["c"].to(a.device, non_blocking=True)
            _mr_start_state(a.xg, req.inputs["lam"], self.dep)
            req.info = _mr_load_step(a, self.dep, c, self.mm.fixed, precision, stream)
            out = torch.empty(a.ndof, dtype=torch.float64, pin_memory=True)
            out.copy_(self.dep, non_blocking=True)
            stream.synchronize()
        req.result = out.numpy()


def _mr_start_state(xg: torch.Tensor, lam: float, dep: torch.Tensor) -> None:
    """The load step's predictor: the affine isochoric stretch z = diag(lam, lam^-1/2, lam^-1/2) x
    with p = 0.  It meets the roller and pulled-face conditions exactly (those boundary nodes are not
    jittered) and keeps every element valid, unlike moving the pulled face alone."""
    nq = xg.shape[1]
    scale = torch.tensor([lam, lam ** -0.5, lam ** -0.5], dtype=xg.dtype, device=xg.device)
    torch.mul(xg, scale[:, None], out=dep[: 3 * nq].view(3, nq))
    dep[3 * nq:] = 0.0


def _mr_load_step(a, dep, c, fixed_u8, precision, stream) -> dict:
    """The request's load step: Newton from `dep` (the predictor, which holds the final Dirichlet
    values) to Iron's default tolerances, consistent tangent, MINRES linear solves."""
    solver = NewtonSolver(a, c, precision=precision, stream=stream)
    info = solver.solve(dep, fixed_u8)[0]
    return {"newton_iterations": info.iterations, "linear_iterations": int(sum(info.linear_iterations)),
            "residual_norm": info.residual_norms[-1], "initial_residual_norm": info.residual_norms[0],
            "reason": info.reason}


# ---- the engine ------------------------------------------------------------------------------------

def estimate_bytes(kind: str, n: int) -> tuple[int, int]:
    """(resident bytes per mesh size, working bytes per request) used for admission: upper
    estimates of the device memory the engine allocates (torch tensors plus the library's
    stream-ordered scratch), so the accounted total never falls below what is in use.  A Laplace
    slot holds laplace_batch_capacity(n) requests' working memory (slot_bytes)."""
    E = n ** 3
    if kind == "laplace":
        N = (n + 1) ** 3
        nnz = (3 * n + 1) ** 3  # exact for the regular trilinear mesh
        resident = 4 * (N + 1) + 4 * nnz + 36 * E + 41 * N
        # + the float-float workspace: coordinates and every element's metrics and matrix
        work = 12 * nnz + 56 * N + 8 * E + 40 * N + 24 * N + 672 * E + 16 * 2048 + 4096
    else:
        Nq, Np = (2 * n + 1) ** 3, (n + 1) ** 3
        ndof = 3 * Nq + Np
        # interior rows: a u node couples with 64 u nodes and 15.6 p nodes on average, a p node
        # with 125 u nodes and 27 p nodes; boundary rows have fewer
        nnz = 3 * Nq * 208 + Np * 402
        resident = 4 * (ndof + 1) + 4 * nnz + 4 * 89 * 89 * E + 4 * (27 + 8 + 89 + 1) * E + 24 * Nq + 10 * ndof
        # values (FP64 + FP32 copy), coordinates, the solution and the Newton vectors, MINRES
        # scratch, the element tangents of a colour batch
        work = 12 * nnz + 24 * Nq + 48 * ndof + 84 * ndof + 27 * 99 * 8 * ((E + 7) // 8)
    return int(1.05 * resident) + (1 << 20), int(1.05 * work) + (1 << 20)


def slot_bytes(kind: str, n: int) -> int:
    """Working bytes charged per Laplace (worker, size) slot or per Mooney-Rivlin request."""
    work = estimate_bytes(kind, n)[1]
    return work * laplace_batch_capacity(n) if kind == "laplace" else work


class HbmLedger:
    """Device-memory bookkeeping of the serving engine (host logic only, no CUDA).

    Charges, against `budget` bytes: resident per-size state (charged when a request for a new size
    is admitted, kept until evicted), Laplace per-(worker, size) slots (kept with their size's
    resident state; a slot serves a batch of up to laplace_batch_capacity(n) requests), and
    Mooney-Rivlin per-request working memory (released when the request ends).  Eviction frees
    least-recently-used sizes that no admitted request holds, together with their slots."""

    def __init__(self, budget: int):
        self.budget = int(budget)
        self.in_use = 0
        self.resident: OrderedDict = OrderedDict()  # (kind, n) -> bytes, LRU order (built or building)
        self.slots: dict = {}  # (worker, kind, n) -> bytes
        self.users: dict = {}  # (kind, n) -> admitted requests holding it
        self.work: dict = {}  # rid -> per-request bytes
        self.evictions = 0

    def _free_for(self, need: int, keep) -> tuple[bool, list, list]:
        evicted, dropped = [], []
        for key in list(self.resident.keys()):
            if self.in_use + need <= self.budget:
                break
            if key == keep or self.users.get(key, 0) > 0:
                continue
            self.in_use -= self.resident.pop(key)
            for sk in [k for k in self.slots if k[1:] == key]:
                self.in_use -= self.slots.pop(sk)
                dropped.append(sk)
            evicted.append(key)
            self.evictions += 1
        return self.in_use + need <= self.budget, evicted, dropped

    def admit(self, rid: int, kind: str, n: int, worker: int):
        """Charge a request; returns (admitted, evicted size keys, dropped slot keys)."""
        key = (kind, n)
        res_b = estimate_bytes(kind, n)[0]
        work_b = slot_bytes(kind, n)
        need = 0 if key in self.resident else res_b
        if kind == "laplace":
            need += 0 if (worker,) + key in self.slots else work_b
        else:
            need += work_b
        ok, evicted, dropped = self._free_for(need, key)
        if not ok:
            return False, evicted, dropped
        if key in self.resident:
            self.resident.move_to_end(key)
        else:
            self.resident[key] = res_b
        if kind == "laplace":
            self.slots.setdefault((worker,) + key, work_b)
        else:
            self.work[rid] = work_b
        self.in_use += need
        self.users[key] = self.users.get(key, 0) + 1
        return True, evicted, dropped

    def finish(self, rid: int, kind: str, n: int) -> None:
        key = (kind, n)
        self.users[key] -= 1
        self.in_use -= self.work.pop(rid, 0)

    def check(self) -> None:
        total = sum(self.resident.values()) + sum(self.slots.values()) + sum(self.work.values())
        assert total == self.in_use, (total, self.in_use)
        assert all(sk[1:] in self.resident for sk in self.slots)


class ServingEngine:
    """Persistent request loop over `workers` CUDA streams with an HBM budget (bytes; default 60 % of
    the free device memory, leaving room for allocator caching and the library's stream-ordered
    scratch, which the estimates do not itemise).  While an engine is alive torch's caching
    allocator is capped at TORCH_MEMORY_FRACTION of the device (lifted by close() of the last
    engine), and a request that runs out of device memory is retried after the engine drains and
    drops its resident state (see serve())."""

    def __init__(self, device=None, workers: int = 8, hbm_budget: int | None = None, use_graphs: bool = True,
                 mr_precision: str = "mixed"):
        self.dev = torch.device(device) if device is not None else _lib.require_cuda()
        _lib.load()
        free, _total = torch.cuda.mem_get_info(self.dev)
        self.ledger = HbmLedger(hbm_budget if hbm_budget is not None else 0.6 * free)
        # torch's caching allocator keeps the blocks of evicted state and finished requests reserved;
        # capped below the device size it releases them before growing further, so the library's
        # stream-ordered scratch (MINRES / CG vectors, outside the ledger) always finds room
        with _ENGINES_LOCK:
            _ENGINES["live"] += 1
            self._closed = False
            torch.cuda.set_per_process_memory_fraction(TORCH_MEMORY_FRACTION, self.dev)
        self.workers = workers
        self.use_graphs = use_graphs
        self.mr_precision = mr_precision
        self.streams = [torch.cuda.Stream(self.dev) for _ in range(workers)]
        # one device error word per worker: a request's kernel errors stay with that request
        self.err_words = [torch.zeros(1, dtype=torch.int32, device=self.dev) for _ in range(workers)]
        self.meshes: dict = {}  # (kind, n) -> resident mesh state
        self.slots: dict = {}  # (worker, "laplace", n) -> slot
        self.lock = threading.Lock()
        self.cv = threading.Condition(self.lock)
        self.stats = {"evictions": 0, "graphs_captured": 0, "max_concurrent": 0, "oom_retries": 0, "batches": 0,
                      "batched_requests": 0}
        self._graveyard: list = []

    @property
    def budget(self) -> int:
        return self.ledger.budget

    @property
    def in_use(self) -> int:
        return self.ledger.in_use

    def _drop(self, evicted, dropped) -> None:
        """Forget evicted state (lock held); slots with graphs are destroyed later, under the
        capture lock."""
        for key in evicted:
            self.meshes.pop(key, None)
        for sk in dropped:
            slot = self.slots.pop(sk, None)
            if slot is not None:
                self._graveyard.append(slot)
        self.stats["evictions"] += len(evicted)

    def _prepare(self, req: Request, worker: int):
        """Resident mesh and, for Laplace, the worker's slot (built on first use, one build at a
        time); a Mooney-Rivlin request gets working buffers of its own."""
        key = (req.kind, req.n)
        sk = (worker,) + key
        with _GRAPH_LOCK:
            with self.lock:
                dead, self._graveyard = self._graveyard, []
                mesh = self.meshes.get(key)
                slot = self.slots.get(sk)
            for d in dead:
                if hasattr(d, "release"):
                    d.release()
            del dead
            if mesh is None:
                mesh = _LaplaceMesh(req.n, self.dev) if req.kind == "laplace" else _MRMesh(req.n, self.dev)
                with self.lock:
                    self.meshes[key] = mesh
            if req.kind == "mr":
                return _MRSlot(mesh, self.dev)
            if slot is None:
                slot = _LaplaceSlot(mesh, self.dev, self.use_graphs)
                slot.capture(self.streams[worker])
                with self.lock:
                    self.stats["graphs_captured"] += slot.n_graphs
                    self.slots[sk] = slot
        return slot

    # run ------------------------------------------------------------------------------------------
    def serve(self, requests: list[Request], realtime: bool = True, log=None) -> dict:
        """Serve `requests` (arrival times in seconds from the start).  With realtime, a request
        is not admitted before its arrival time.  Returns summary statistics; per-request results
        and times are stored on the requests.  Raises GfeError after the running requests have
        finished if a request failed or cannot fit the budget at all.

        A request that runs out of device memory (the ledger's estimates do not see the caching
        allocator's fragmentation) goes back to the head of the queue: the engine admits nothing
        until the running requests have finished, drops its resident state, returns the
        allocator's cached blocks and admits again; a request that fails that way OOM_RETRIES
        times is an error."""
        order = sorted(requests, key=lambda r: r.arrival)
        pending: deque = deque()
        free_workers = list(range(self.workers))
        running = 0
        errors = []
        retries: dict = {}
        compact = [False]
        t0 = time.perf_counter()
        clock = (lambda: time.perf_counter() - t0) if realtime else (lambda: math.inf)
        nxt = 0
        done_count = 0
        fatal = None

        def work(group: list, worker: int):
            nonlocal running, done_count
            stream = self.streams[worker]
            lead = group[0]
            try:
                _lib.set_thread_error_word(self.err_words[worker])
                with torch.cuda.stream(stream):
                    slots = [self._prepare(r, worker) for r in group]
                slot = slots[0]
                del slots
                if lead.kind == "laplace":
                    before = slot.n_graphs
                    slot.run(group, stream)
                    with self.lock:
                        self.stats["graphs_captured"] += slot.n_graphs - before
                else:
                    slot.run(lead, stream, self.mr_precision)
                    del slot  # per-request working memory
            except Exception as e:  # reported after the loop
                oom = _is_out_of_memory(e) and all(retries.get(r.rid, 0) < OOM_RETRIES for r in group)
                if not oom:
                    errors.extend((r.rid, repr(e)) for r in group)
            else:
                oom = False
            finally:
                t_done = time.perf_counter() - t0
                with self.cv:
                    running -= 1
                    for r in group:
                        r.t_done = t_done
                        self.ledger.finish(r.rid, r.kind, r.n)
                    free_workers.append(worker)
                    if oom:
                        # retried alone, at the head of the queue
                        for r in reversed(group):
                            retries[r.rid] = retries.get(r.rid, 0) + 1
                            pending.appendleft(r)
                        compact[0] = True
                        self.stats["oom_retries"] += 1
                    else:
                        done_count += len(group)
                    self.cv.notify_all()

        threads = []
        with self.cv:
            while done_count < len(order) and fatal is None:
                now = clock()
                while nxt < len(order) and order[nxt].arrival <= now:
                    pending.append(order[nxt])
                    nxt += 1
                if compact[0]:
                    if running > 0:
                        self.cv.wait(timeout=0.5)
                        continue
                    # nothing in flight: drop the resident state too (its blocks pin the fragmented
                    # segments) and return every cached block before admitting again.  The engine
                    # lock is released meanwhile (the reset takes the capture lock first).
                    self.cv.release()
                    try:
                        self._reset_resident()
                    finally:
                        self.cv.acquire()
                    compact[0] = False
                # requests withdrawn while queued are dropped without running
                for req in [r for r in pending if r.cancelled]:
                    pending.remove(req)
                    done_count += 1
                # admit in arrival order; a request that does not fit may be overtaken.  A small
                # Laplace request takes queued requests of its side along (up to the slot's
                # capacity), except one that is being retried after running out of memory
                i = 0
                while i < len(pending) and free_workers:
                    req = pending[i]
                    w = free_workers[-1]
                    ok, evicted, dropped = self.ledger.admit(req.rid, req.kind, req.n, w)
                    self._drop(evicted, dropped)
                    if ok:
                        free_workers.pop()
                        del pending[i]
                        group = [req]
                        if req.kind == "laplace" and req.rid not in retries:
                            cap = laplace_batch_capacity(req.n)
                            j = i
                            while len(group) < cap and j < len(pending):
                                r = pending[j]
                                if (r.kind == "laplace" and r.n == req.n and r.rid not in retries
                                        and self.ledger.admit(r.rid, r.kind, r.n, w)[0]):
                                    group.append(r)
                                    del pending[j]
                                else:
                                    j += 1
                        now = clock() if realtime else time.perf_counter() - t0
                        for r in group:
                            r.t_admit = now
                        if len(group) > 1:
                            self.stats["batches"] += 1
                            self.stats["batched_requests"] += len(group)
                        running += 1
                        self.stats["max_concurrent"] = max(self.stats["max_concurrent"], running)
                        th = threading.Thread(target=work, args=(group, w), daemon=True)
                        threads.append(th)
                        th.start()
                    else:
                        i += 1
                if pending and running == 0:
                    # nothing running and the head still does not fit: the budget is too small
                    req = pending[0]
                    fatal = GfeError(-7, f"request {req.rid} ({req.kind} n={req.n}) does not fit the HBM budget "
                                         f"of {self.budget} bytes")
                    break
                if done_count >= len(order):
                    break
                wait = None
                if nxt < len(order) and realtime:
                    wait = max(0.0, order[nxt].arrival - clock())
                self.cv.wait(timeout=wait if wait is not None else 0.5)
        for th in threads:
            th.join()
        if fatal is not None:
            raise fatal
        if errors:
            raise GfeError(-4, f"{len(errors)} request(s) failed, first: {errors[0]}")
        return summarize(order)

    def close(self):
        """Drop every resident mesh and slot, return the cached blocks to the device and lift the
        engine's cap on torch's allocator once no other engine is alive."""
        if getattr(self, "_closed", True):
            return
        self._reset_resident()
        with _ENGINES_LOCK:
            self._closed = True
            _ENGINES["live"] -= 1
            if _ENGINES["live"] == 0:
                torch.cuda.set_per_process_memory_fraction(1.0, self.dev)

    def _reset_resident(self):
        """Drop every resident mesh and slot (graphs are destroyed under the capture lock) and
        return the allocator's cached blocks to the device.  No request may be running."""
        with _GRAPH_LOCK:
            with self.lock:
                dead = list(self.slots.values()) + self._graveyard
                self.slots.clear()
                self.meshes.clear()
                self._graveyard = []
                self.ledger = HbmLedger(self.ledger.budget)
            for slot in dead:
                if hasattr(slot, "release"):
                    slot.release()
            del dead
        torch.cuda.synchronize(self.dev)
        torch.cuda.empty_cache()
        with torch.cuda.device(self.dev):
            _lib.call("gfe_release_scratch")  # the library's cached stream-ordered scratch too

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def summarize(reqs: list[Request]) -> dict:
    cancelled = sum(1 for r in reqs if r.cancelled and math.isnan(r.t_admit))
    reqs = [r for r in reqs if not (r.cancelled and math.isnan(r.t_admit))]
    if not reqs:
        return {"requests": 0, "cancelled": cancelled}
    lat = np.array([r.latency for r in reqs]) * 1e3
    t_end = max(r.t_done for r in reqs)
    t_first = min(r.arrival for r in reqs)
    span = t_end - t_first
    E = sum(r.elements for r in reqs)
    out = {"requests": len(reqs), "cancelled": cancelled,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "span_s": span,
           "requests_per_s": len(reqs) / span, "elements_per_s": E / span}
    for kind in ("laplace", "mr"):
        rk = [r for r in reqs if r.kind == kind]
        if not rk:
            continue
        lk = np.array([r.latency for r in rk]) * 1e3
        sk = np.array([r.t_done - r.t_admit for r in rk]) * 1e3
        out[f"{kind}_p50_ms"] = float(np.percentile(lk, 50))
        out[f"{kind}_p99_ms"] = float(np.percentile(lk, 99))
        out[f"{kind}_service_mean_ms"] = float(sk.mean())
        its = [r.info.get("linear_iterations", r.info.get("iterations")) for r in rk]
        its = [i for i in its if i is not None]
        if its:
            out[f"{kind}_solver_iterations_mean"] = float(np.mean(its))
        nits = [r.info["newton_iterations"] for r in rk if "newton_iterations" in r.info]
        if nits:
            out[f"{kind}_newton_iterations_mean"] = float(np.mean(nits))
        batch = [r.info["batch"] for r in rk if "batch" in r.info]
        if batch:
            out[f"{kind}_batch_mean"] = float(np.mean(batch))
    return out


# ---- the baseline: the plain FP64 path, one request at a time ------------------------------------

def plain_fp64(requests: list[Request], realtime: bool = True) -> dict:
    """Each request from scratch (mesh, structure, FP64 colour-scatter assembly, FP64 solve), one
    at a time in arrival order, on the default stream."""
    order = sorted(requests, key=lambda r: r.arrival)
    dev = _lib.require_cuda()
    t0 = time.perf_counter()
    for req in order:
        if realtime:
            wait = req.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        req.t_admit = time.perf_counter() - t0
        if req.kind == "laplace":
            m = RegularMesh((req.n,) * 3)
            A = LaplaceAssembly(m.elem_nodes, req.inputs["coords"].numpy(), kappa=req.inputs["kappa"].numpy(),
                                colour_elems=m.colouring()[0], colour_ptr=m.colouring()[1], device=dev)
            A.assemble("fp64", path="general")
            fixed, x0 = _laplace_bcs(m)
            x = torch.from_numpy(x0).to(dev)
            info = A.solve(torch.from_numpy(fixed).to(dev), x, rtol=LAPLACE_RTOL, precision="fp64")
            req.result = x.cpu().numpy()
            req.info = {"iterations": info.iterations, "rel_residual": info.relative_residual}
        else:
            m = RegularMesh((req.n,) * 3, order=2)
            elin, lin2g = linear_component(m.elem_nodes, 2)
            order_c, ptr = m.colouring()
            A = MooneyRivlinAssembly(m.elem_nodes, elin, req.inputs["coords"].numpy(), order_c, ptr, len(lin2g),
                                     device=dev)
            c = req.inputs["c"].to(dev)
            fixed, _full = uniaxial_roller_conditions(A, req.inputs["lam"])
            dep = torch.empty(A.ndof, dtype=torch.float64, device=dev)
            _mr_start_state(A.xg, req.inputs["lam"], dep)
            req.info = _mr_load_step(A, dep, c, fixed, "fp64", None)
            req.result = dep.cpu().numpy()
        torch.cuda.synchronize()
        req.t_done = time.perf_counter() - t0
    return summarize(order)


# ---- bench entry -----------------------------------------------------------------------------------

def _agreement(reqs, res_engine) -> dict:
    """Engine results against the plain FP64 path's (on the requests): Laplace solutions (both CG
    to a relative residual of 1e-10); Mooney-Rivlin geometry and pressure (both Newton to Iron's
    tolerances, FP32 contraction and Krylov in the engine, FP64 in the plain path)."""
    lap, mr_x, mr_p = 0.0, 0.0, 0.0
    for r in reqs:
        a, b = res_engine[r.rid], r.result
        if r.kind == "laplace":
            lap = max(lap, float(np.abs(a - b).max()))
        else:
            nx = 3 * (2 * r.n + 1) ** 3
            mr_x = max(mr_x, float(np.abs(a[:nx] - b[:nx]).max()))
            mr_p = max(mr_p, float(np.abs(a[nx:] - b[nx:]).max() / max(np.abs(b[nx:]).max(), 1e-300)))
    return {"laplace_max_abs_diff_vs_plain": lap, "mr_geometry_max_abs_diff_vs_plain": mr_x,
            "mr_pressure_max_rel_diff_vs_plain": mr_p}


def measure_stream(reqs: list[Request], workers: int, clock_sampler, log) -> dict:
    """Serve `reqs` in real time through a fresh engine, then through plain_fp64 one at a time
    (on an empty device), and compare.  Inputs must be made; a small warm-up stream runs first."""
    dev = torch.device("cuda", 0)
    eng = ServingEngine(dev, workers=workers)
    # warm-up of both arms: small requests of each kind (library load and page-in, kernel attributes)
    warm = request_stream(n_requests=4, laplace_fraction=0.5, seed=99, n_lo=4, n_hi=5)
    assert {r.kind for r in warm} == {"laplace", "mr"}
    for r in warm:
        make_inputs(r)
    eng.serve(warm, realtime=False)
    for r in warm:
        r.result = None
    plain_fp64(warm, realtime=False)
    log(f"serve: engine, {len(reqs)} requests")
    with clock_sampler(dev.index) as clk:
        s_eng = eng.serve(reqs, realtime=True)
    res_engine = {r.rid: r.result for r in reqs}
    log(f"serve: engine p50 {s_eng['p50_ms']:.1f} ms p99 {s_eng['p99_ms']:.1f} ms; plain FP64 baseline")
    engine_stats = dict(eng.stats)
    budget = eng.budget
    eng.close()  # the plain path runs on an empty device, as a process of its own would
    for r in reqs:
        r.result = None
    with clock_sampler(dev.index) as clk2:
        s_plain = plain_fp64(reqs, realtime=True)
    out = {"engine": s_eng, "plain_fp64_one_at_a_time": s_plain,
           "p50_speedup_vs_plain": s_plain["p50_ms"] / s_eng["p50_ms"],
           "p99_speedup_vs_plain": s_plain["p99_ms"] / s_eng["p99_ms"],
           "throughput_speedup_vs_plain": s_eng["requests_per_s"] / s_plain["requests_per_s"]}
    out.update(_agreement(reqs, res_engine))
    out.update({"engine_stats": engine_stats, "hbm_budget_GB": budget / 1e9, "clocks": clk.summary(),
                "clocks_plain": clk2.summary()})
    if _lib.STALE_ERRORS:
        out["stale_cuda_errors"] = {f"{k[0]}:{k[1]}": v for k, v in _lib.STALE_ERRORS.items()}
    return out


def stream_config(reqs: list[Request], rate: float, n_hi: int, mr_n_hi: int, workers: int) -> dict:
    return {"workload": "serve_stream", "requests": len(reqs), "arrivals": f"Poisson {rate:g}/s", "laplace": 0.7,
            "side": f"round(exp(U(ln 4, ln {n_hi})))", "mr_side": f"round(exp(U(ln 4, ln {mr_n_hi})))",
            "laplace_solve": f"CG rtol {LAPLACE_RTOL}",
            "mr_solve": "one load step: Newton to abs 1e-10 / rel 1e-5 (step 1e-5), MINRES rtol 1e-5",
            "batching": f"up to {LAPLACE_BATCH} Laplace requests of one side <= {BATCH_MAX_N} per graph launch",
            "workers": workers}


# Mooney-Rivlin sides of the served streams: a Newton load step at side 64 (6.7 M unknowns) takes
# the order of a minute on one GPU, so served Mooney-Rivlin requests stay at sides 4..MR_SERVE_N_HI
MR_SERVE_N_HI = 16


def bench(args, log, clock_sampler):
    """The request-stream workload: Poisson arrivals at 200/s (sides 4..64, Mooney-Rivlin sides
    4..MR_SERVE_N_HI), served by the engine and by the plain path."""
    import json

    n_req = getattr(args, "serve_requests", 2000)
    rate = getattr(args, "serve_rate", 200.0)
    workers = getattr(args, "serve_workers", 8)
    reqs = request_stream(n_requests=n_req, rate=rate, seed=0, mr_n_hi=MR_SERVE_N_HI)
    log(f"serve: generating inputs for {len(reqs)} requests")
    for r in reqs:
        make_inputs(r)
    m = measure_stream(reqs, workers, clock_sampler, log)
    line = {
        "metric": "serve_p99_latency_ms", "value": m["engine"]["p99_ms"], "unit": "ms", "n_gpus": 1, "steps": 1,
        "warmup": 1, "higher_is_better": False, "dtype": "f64 (Laplace mixed_df assembly), f32/f64 (MR)",
        "data": "synthetic", "config": stream_config(reqs, rate, 64, MR_SERVE_N_HI, workers),
    }
    line.update(m)
    print(json.dumps(line), flush=True)
    return 0
