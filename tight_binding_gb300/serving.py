"""Many density-of-states solves advanced together (libtbk ``tbk_server_*``).

The reference runs one solve per call (``density_of_states_seq``,
TB/functions.h:15-32).  :class:`DosServer` takes a stream of requests — a
lattice, spectral bounds, number of moments M, random vectors R, seed and
precision — and returns each request's Chebyshev moments mu_0 .. mu_{M-1}
(those of ``KpmSolver.run_device`` with doubling and the same seed).  Requests
are admitted against an HBM budget, built on the device, and advanced in rounds
of CUDA-graph-captured recursion steps packed over all running requests.  A
request gives the same bits alone and in any mix.
"""
from __future__ import annotations

import ctypes as C
import time
from typing import Sequence

import numpy as np

from . import capi
from .capi import check, lib
from .lattice import PartialLattice

# lattices of the serving workload: nearest-neighbour hopping from every atom
# (TB/models.h:5-151 cells), coordination number for the spectral bounds
MODEL_ATOMS = {"square": ("A",), "honeycomb": ("A", "B"), "kagome": ("A", "B", "C"), "lieb": ("A", "B", "C"),
               "fcc": ("A",)}
MODEL_COORD = {"square": 4, "honeycomb": 3, "kagome": 4, "lieb": 4, "fcc": 12}


def model_cell(kind: str, t: float = 1.0):
    """Unit cell of `kind` with nearest-neighbour hopping t from every atom (the
    h.c. duplicates that later atoms would add are skipped, as the reference's
    add_hopping does)."""
    from . import lattice as lat
    c = {"square": lat.Square, "honeycomb": lat.Honeycomb, "kagome": lat.Kagome, "lieb": lat.Lieb,
         "fcc": lat.FCC}[kind]()
    for a in MODEL_ATOMS[kind]:
        c.add_hopping(a, 1, t)
    return c


def model_bounds(kind: str, W: float, t: float = 1.0, margin: float = 0.05) -> tuple[float, float]:
    """Symmetric spectral bounds z|t| + W/2 + margin for on-site disorder U[-W/2, W/2]."""
    e = MODEL_COORD[kind] * abs(t) + W / 2 + margin
    return -e, e


PRECISION = {"mixed": capi.PREC_MIXED, "fp64": capi.PREC_FP64, "dd": capi.PREC_DD}
MODES = {"periodic": capi.BUILD_PERIODIC_BARE, "open": capi.BUILD_SPARSE, "bare": capi.BUILD_BARE}
STATS_KEYS = ("done", "failed", "rounds", "graphs", "busy_ms", "bytes", "updates", "launches", "budget_bytes",
              "peak_reserved_bytes", "reserved_bytes", "build_ms", "peak_resident", "build_overshoot_bytes")


def _request(lattice: PartialLattice, n_mom: int, R: int, seed: int, e_min: float, e_max: float,
             precision: str = "mixed", mode: str = "periodic", extend: Sequence[int] | None = None,
             scalar=float) -> capi.Request:
    q = capi.Request()
    q.lattice = lattice._h
    q.build_mode = MODES[mode]
    ext = [1] * lattice.dim if extend is None else list(extend)
    ext = ext[:lattice.dim] + [0] * (3 - lattice.dim)
    for i in range(3):
        q.extend[i] = int(ext[i])
    q.is_complex = 1 if scalar is complex else 0
    q.n_mom = int(n_mom)
    q.R = int(R)
    q.precision = PRECISION[precision]
    q.seed = int(seed)
    q.e_min = float(e_min)
    q.e_max = float(e_max)
    return q


KINDS = {"dos": capi.REQ_DOS, "bastin": capi.REQ_KUBO_BASTIN, "greenwood": capi.REQ_KUBO_GREENWOOD}


def request_footprint(lattice: PartialLattice, n_mom: int, R: int, precision: str = "mixed",
                      e_min: float = -1.0, e_max: float = 1.0, kind: str = "dos", axes=(0, 1),
                      **kw) -> tuple[int, int]:
    """(build peak bytes, resident bytes) that admission charges for a request
    (conductivity kinds: at the 120 GB default budget)."""
    q = _request(lattice, n_mom, R, 0, e_min, e_max, precision, **kw)
    q.kind = KINDS[kind]
    if kind != "dos":
        q.axis[0], q.axis[1] = int(axes[0]), int(axes[1] if len(axes) > 1 else axes[0])
        q.kernel = capi.KERNEL_LORENTZ
    peak, res = C.c_int64(), C.c_int64()
    check(lib().tbk_request_footprint(C.byref(q), C.byref(peak), C.byref(res)))
    return int(peak.value), int(res.value)


class DosServer:
    """Continuous-batching server of DoS moment requests on one GPU; it also
    takes conductivity (Kubo mu_nm) requests, which run as one solve each on
    the admission stream while the DoS rounds go on."""

    def __init__(self, budget_gb: float = 120.0, steps_per_round: int = 16, autotune: bool = True,
                 max_resident: int = 4096, result_arena_mb: int = 64, step_gb: float = 2.0):
        cfg = capi.ServerConfig(float(budget_gb), int(steps_per_round), 1 if autotune else 0, int(max_resident),
                                int(result_arena_mb), float(step_gb))
        h = C.c_void_p()
        check(lib().tbk_server_create(C.byref(h), C.byref(cfg)))
        self._h = h
        self._n_mom: dict[int, int] = {}
        self._kubo: set[int] = set()

    def submit(self, lattice: PartialLattice, n_mom: int, R: int, seed: int, e_min: float, e_max: float,
               precision: str = "mixed", mode: str = "periodic", extend: Sequence[int] | None = None,
               scalar=float) -> int:
        """Queues a request (the lattice is copied); returns its ticket."""
        q = _request(lattice, n_mom, R, seed, e_min, e_max, precision, mode, extend, scalar)
        t = C.c_int64()
        check(lib().tbk_server_submit(self._h, C.byref(q), C.byref(t)))
        self._n_mom[t.value] = int(n_mom)
        return int(t.value)

    def submit_kubo(self, lattice: PartialLattice, kind: str, M: int, R: int, seed: int, e_min: float,
                    e_max: float, axes=(0, 1), kernel=None, precision: str = "dd", mode: str = "periodic",
                    extend: Sequence[int] | None = None, scalar=complex) -> int:
        """Queues a conductivity request; poll returns g_m g_n mu_nm (M x M complex).
        kind "bastin": mu_nm = <T_m r | v_a T_n v_b r> (conductivity_Kubo_Bastin);
        "greenwood": mu_nm = <v_a T_m v_a r | T_n r> (conductivity_spectrum);
        v_a = [x_a, H~] with H~ = (H - b)/a from e_min, e_max."""
        from .kpm import Lorentz
        kernel = kernel if kernel is not None else Lorentz(6.0)
        q = _request(lattice, M, R, seed, e_min, e_max, precision, mode, extend, scalar)
        q.kind = {"bastin": capi.REQ_KUBO_BASTIN, "greenwood": capi.REQ_KUBO_GREENWOOD}[kind]
        q.axis[0], q.axis[1] = int(axes[0]), int(axes[1] if len(axes) > 1 else axes[0])
        q.kernel, q.kernel_p0, q.kernel_p1 = kernel.kind, float(kernel.p0), float(kernel.p1)
        t = C.c_int64()
        check(lib().tbk_server_submit(self._h, C.byref(q), C.byref(t)))
        self._n_mom[t.value] = int(M)
        self._kubo.add(t.value)
        return int(t.value)

    def poll(self, ticket: int, wait_ms: int = 0):
        """(mu, times_ms) when done, None while pending; raises TbkError if it failed.
        times_ms = [queued, build, resident, total].  Kubo requests: mu is the
        M x M complex mu_nm."""
        n = self._n_mom[ticket]
        kubo = ticket in self._kubo
        mu = np.empty(2 * n * n if kubo else n, dtype=np.float64)
        times = np.zeros(4, dtype=np.float64)
        s = lib().tbk_server_poll(self._h, int(ticket), int(wait_ms), capi.ptr(mu), capi.ptr(times))
        if s == capi.TBK_PENDING:
            return None
        self._n_mom.pop(ticket, None)
        self._kubo.discard(ticket)
        check(s)
        if kubo:
            mu = mu.view(np.complex128).reshape(n, n)
        return mu, times

    def result(self, ticket: int, timeout_s: float = 600.0):
        """Blocks until the request is done (bounded by timeout_s)."""
        t_end = time.monotonic() + timeout_s
        while True:
            r = self.poll(ticket, 100)
            if r is not None:
                return r
            if time.monotonic() > t_end:
                raise TimeoutError(f"request {ticket} not done after {timeout_s} s")

    def stats(self) -> dict:
        v = np.zeros(len(STATS_KEYS), dtype=np.float64)
        check(lib().tbk_server_stats(self._h, capi.ptr(v), len(STATS_KEYS)))
        return dict(zip(STATS_KEYS, v.tolist()))

    def tuning(self) -> list[dict]:
        rows = np.zeros((128, 6), dtype=np.float64)
        k = lib().tbk_server_tuning(self._h, 128, capi.ptr(rows))
        names = {capi.PREC_MIXED: "mixed", capi.PREC_FP64: "fp64", capi.PREC_DD: "dd"}
        return [dict(precision=names.get(int(r[0]), str(int(r[0]))), width=int(r[1]),
                     form="classes" if int(r[2]) else "ell", grid=int(r[3]), prefetch=int(r[4]),
                     ms_per_step=float(r[5])) for r in rows[:max(k, 0)]]

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().tbk_server_destroy(h)
        self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
