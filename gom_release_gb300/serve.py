"""Serving storm-surge runs on one GPU: continuous batching.

A request is one storm-surge run (mesh, storm, horizon).  ``PackedServer`` (the serving form)
keeps every in-flight run in one packed context, so each phase of a step is one launch over all
runs; ``Server`` keeps one context per run and steps them in turn each tick.  Both retire runs
that reach their horizon and admit waiting requests when the device-memory budget has room (the
device bytes of new work are estimated from the bytes per cell-layer of the contexts created so
far).

``serve_fifo`` is the comparison the configuration asks for: the same requests served one at a
time, in arrival order, each run to its horizon before the next starts.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from .core import GomCore, GomError
from .deck import Deck


@dataclasses.dataclass(eq=False)
class Request:
    rid: int
    deck: Deck                # mesh + parameters (precision set by the server)
    storm: object             # gom_storm fields
    steps: int                # horizon in timesteps
    arrival: float            # seconds after the start of the stream
    cell_layers: int = 0      # active cell-layers at the start (work per step)
    started: float = -1.0
    finished: float = -1.0
    done_steps: int = 0
    error: str = ""
    t0: float = 0.0           # context clock at which the run started (packed serving)


def storm_context(lib, deck: Deck, precision: int, storms: list) -> GomCore:
    """A context for a storm-surge deck (one run or a packed ensemble, one storm per run) with
    its initial state and forcing set up on the device."""
    d = dataclasses.replace(deck, params=dataclasses.replace(deck.params, precision=precision))
    c = GomCore(d, lib=lib)
    p = d.params
    c.cold_start(p.ref_salt, p.ref_temp, p.av_0, p.kv_0)
    c.step("density")
    nt = max(1, p.trans_sub_iter)
    cob = np.zeros((d.n_ob, 2, nt))
    cob[:, 0, :] = p.ref_salt
    cob[:, 1, :] = p.ref_temp
    c.set_forcing({"elapsed_time": 0.0, "spinup_tide": 1.0, "spinup_baroclinic": 1.0, "con_at_ob": cob})
    c.set_storms(storms, elapsed_time=0.0)
    return c


def active_cell_layers(core: GomCore, deck: Deck) -> int:
    top = core.get_field("top_layer_cell")
    bot = deck.geo["bottom_layer_at_element"]
    wet = top > 0
    return int(np.sum(top[wet] - bot[wet] + 1))


class Server:
    """Continuous batching of storm-surge runs under a device-memory budget."""

    def __init__(self, lib, budget_bytes: float, precision: int = 1, on_finish=None):
        self.lib = lib
        self.on_finish = on_finish         # called with (request, context) before a run is retired
        self.budget = float(budget_bytes)
        self.precision = precision
        self.active: list[tuple[Request, GomCore]] = []
        self.waiting: list[Request] = []
        self.used = 0.0
        self.bytes_per_cell_layer = None   # learned from created contexts
        self.peak_bytes = 0.0
        self.peak_active = 0

    def _estimate(self, req: Request) -> float:
        cl = req.deck.n_cells * (req.deck.n_layers + 2)
        return cl * (self.bytes_per_cell_layer or 0.0)

    def admit(self, now: float):
        while self.waiting:
            req = self.waiting[0]
            if self.active and self.used + self._estimate(req) > self.budget:
                return
            self.waiting.pop(0)
            core = storm_context(self.lib, req.deck, self.precision, [req.storm])
            nbytes = core.device_bytes()
            self.bytes_per_cell_layer = max(self.bytes_per_cell_layer or 0.0,
                                            nbytes / (req.deck.n_cells * (req.deck.n_layers + 2)))
            req.cell_layers = active_cell_layers(core, req.deck)
            req.started = now
            self.used += nbytes
            self.peak_bytes = max(self.peak_bytes, self.used)
            self.active.append((req, core))
            self.peak_active = max(self.peak_active, len(self.active))

    def tick(self, clock) -> list[Request]:
        # Contexts are stepped one after another: the free-surface solve is a cooperative kernel
        # that spins on grid barriers, and with the steps of many contexts queued on concurrent
        # streams the block scheduler may keep its remaining blocks waiting behind other streams'
        # kernels past the barrier's time limit (measured: GOM_E_TIMEOUT with 13 contexts in
        # flight).  Device-side overlap of many runs is what PackedServer provides.
        failed = set()
        for req, core in self.active:
            try:
                core.step_launch()
                core.step_wait()
            except GomError as e:      # a run that stops (as the reference would) leaves the mix
                req.error = str(e)
                failed.add(req.rid)
        now = clock()
        done, keep = [], []
        for req, core in self.active:
            req.done_steps += 1
            if req.done_steps >= req.steps or req.rid in failed:
                req.finished = now
                if self.on_finish:
                    self.on_finish(req, core)
                self.used -= core.device_bytes()
                core.close()
                done.append(req)
            else:
                keep.append((req, core))
        self.active = keep
        return done


def serve(lib, requests: list[Request], budget_bytes: float, precision: int = 1) -> dict:
    """Replay a request stream in wall time; returns per-request latency and totals."""
    srv = Server(lib, budget_bytes, precision)
    pending = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    clock = lambda: time.perf_counter() - t0  # noqa: E731
    finished: list[Request] = []
    i = 0
    work = 0
    while len(finished) < len(requests):
        now = clock()
        while i < len(pending) and pending[i].arrival <= now:
            srv.waiting.append(pending[i])
            i += 1
        srv.admit(now)
        if not srv.active:
            if i < len(pending):
                time.sleep(max(0.0, min(0.01, pending[i].arrival - now)))
            continue
        work += sum(r.cell_layers for r, _ in srv.active)
        finished += srv.tick(clock)
    wall = clock()
    return _summary(requests, wall, work, srv.peak_bytes, srv.peak_active)


def serve_fifo(lib, requests: list[Request], precision: int = 0) -> dict:
    """The same requests served one at a time in arrival order."""
    pending = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    clock = lambda: time.perf_counter() - t0  # noqa: E731
    work = 0
    peak = 0.0
    for req in pending:
        now = clock()
        if now < req.arrival:
            time.sleep(req.arrival - now)
        core = storm_context(lib, req.deck, precision, [req.storm])
        peak = max(peak, core.device_bytes())
        req.cell_layers = active_cell_layers(core, req.deck)
        req.started = clock()
        try:
            for _ in range(req.steps):
                core.step_launch()
                core.step_wait()
        except GomError as e:
            req.error = str(e)
        req.finished = clock()
        req.done_steps = req.steps
        work += req.cell_layers * req.steps
        core.close()
    return _summary(requests, clock(), work, peak, 1)


def _summary(requests, wall, work, peak_bytes, peak_active) -> dict:
    lat = np.array([r.finished - r.arrival for r in requests])
    return {"requests": len(requests), "failed": sum(1 for r in requests if r.error),
            "errors": sorted({r.error for r in requests if r.error}), "wall_s": wall,
            "cell_layer_steps": int(work),
            "throughput": work / wall if wall > 0 else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_mean_s": float(lat.mean()), "peak_device_bytes": float(peak_bytes),
            "peak_in_flight": int(peak_active)}


def poisson_arrivals(n: int, rate: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


__all__ = ["Request", "Server", "PackedServer", "serve", "serve_packed", "serve_fifo", "poisson_arrivals",
           "active_cell_layers", "storm_context"]


class PackedServer:
    """Continuous batching with every in-flight run packed into one context: each phase of a step
    is one launch over all runs (per-run PCG), and the storms are evaluated on the device with a
    clock offset per run.  Requests that arrive while others run are admitted at the next repack:
    a new packed context is created with the runs still in flight plus the newcomers, the in-flight
    runs' state is copied over with gom_copy_run, the newcomers start from a device cold start.
    Repacks happen when requests are waiting (at most every ``min_interval`` seconds), when
    finished runs hold more than half of the packed cells, or when a run has failed.

    Memory: a repack holds the old and the new context at once, so a request is admitted only
    while the old context's bytes plus the new pack's estimated bytes fit the budget; the bytes per
    cell-layer are measured on a one-run context before the first admission and refined from
    every pack created.  ``peak_bytes`` counts that transient.

    Failures: the device reports the first failing entity of a step and the library maps it to its
    run (gom_status.run).  Only that run is retired with the error; the step completed for the
    others (their phases never read another run's values), which continue in the next pack.  A
    failure that names no run (a solver barrier that timed out) fails every run of the pack."""

    def __init__(self, lib, budget_bytes: float, precision: int = 1, min_interval: float = 0.5,
                 on_finish=None):
        self.lib = lib
        self.budget = float(budget_bytes)
        self.precision = precision
        self.min_interval = min_interval
        self.on_finish = on_finish
        self.core: GomCore | None = None
        self.deck: Deck | None = None
        self.members: list[Request] = []      # run r of the current pack is members[r]
        self.waiting: list[Request] = []
        self.elapsed = 0.0                    # context clock (s of simulated time)
        self.last_repack = -1e30
        self.bytes_per_cell_layer = None
        self.peak_bytes = 0.0
        self.peak_active = 0
        self.repacks = 0
        self.repack_s: list[float] = []       # wall seconds of every repack
        self.failed_runs = 0
        self.rejected: list[Request] = []     # requests larger than the whole budget
        self._gc_now = False                  # a run failed: drop it at the next repack

    def _cells(self, reqs) -> float:
        return float(sum(r.deck.n_cells * (r.deck.n_layers + 2) for r in reqs))

    def active(self) -> list[Request]:
        return [r for r in self.members if r.finished < 0]

    def _measure_bytes_per_cell_layer(self, req: Request) -> float:
        """Device bytes per cell-layer of a one-run context of ``req`` (created and closed)."""
        c = storm_context(self.lib, req.deck, self.precision, [req.storm])
        try:
            return c.device_bytes() / self._cells([req])
        finally:
            c.close()

    def maybe_repack(self, now: float):
        live = self.active()
        dead = self._cells([r for r in self.members if r.finished >= 0])
        want_new = bool(self.waiting) and (now - self.last_repack >= self.min_interval or not live)
        want_gc = self._gc_now or dead > 0.5 * max(self._cells(self.members), 1.0)
        if not (want_new or want_gc):
            return
        old_bytes = float(self.core.device_bytes()) if self.core is not None else 0.0
        admitted = []
        if want_new:
            if self.bytes_per_cell_layer is None:
                self.bytes_per_cell_layer = self._measure_bytes_per_cell_layer(self.waiting[0])
            bpcl = self.bytes_per_cell_layer
            used = self._cells(live)
            # the old context stays alive while the new one is filled
            while self.waiting and old_bytes + bpcl * (used + self._cells([self.waiting[0]])) <= self.budget:
                r = self.waiting.pop(0)
                used += self._cells([r])
                admitted.append(r)
            if not admitted and not live and self.waiting:
                # nothing in flight and the first request alone exceeds the budget: it cannot run
                r = self.waiting.pop(0)
                r.error = "request exceeds the device-memory budget"
                r.started = r.finished = now
                r.done_steps = 0
                self.rejected.append(r)
        if not admitted and not want_gc:
            return
        if (not admitted and live and self.bytes_per_cell_layer
                and old_bytes + self.bytes_per_cell_layer * self._cells(live) > self.budget):
            return   # the shrunk pack does not fit beside the old one yet; wait for runs to finish
        self._gc_now = False
        self._repack(live, admitted, now, old_bytes)

    def _repack(self, live, admitted, now, old_bytes=0.0):
        from .ensemble import pack
        t_start = time.perf_counter()
        old, old_members = self.core, self.members
        members = live + admitted
        self.members = members
        self.last_repack = now
        self.repacks += 1
        if not members:
            if old is not None:
                old.close()
            self.core = None
            self.repack_s.append(time.perf_counter() - t_start)
            return
        base = pack([r.deck for r in members])
        deck = dataclasses.replace(base, params=dataclasses.replace(base.params, precision=self.precision))
        core = GomCore(deck, lib=self.lib)
        p = deck.params
        core.cold_start(p.ref_salt, p.ref_temp, p.av_0, p.kv_0)
        core.step("density")
        nt = max(1, p.trans_sub_iter)
        cob = np.zeros((deck.n_ob, 2, nt))
        cob[:, 0, :] = p.ref_salt
        cob[:, 1, :] = p.ref_temp
        core.set_forcing({"elapsed_time": self.elapsed, "spinup_tide": 1.0, "spinup_baroclinic": 1.0,
                          "con_at_ob": cob})
        for r in admitted:
            r.t0 = self.elapsed
            r.started = now
        core.set_storms([dataclasses.replace(r.storm, t0=r.t0) for r in members], elapsed_time=self.elapsed)
        nbytes = core.device_bytes()
        self.peak_bytes = max(self.peak_bytes, float(nbytes) + old_bytes)   # both contexts are alive here
        if old is not None:
            for new_idx, r in enumerate(live):
                core.copy_run(new_idx, old, old_members.index(r))
            old.close()
        top = core.get_field("top_layer_cell")
        bot = deck.geo["bottom_layer_at_element"]
        cs = deck.runs["run_cell_start"]
        for i, r in enumerate(members):
            if r in admitted:
                sl = slice(cs[i], cs[i + 1])
                t, b = top[sl], bot[sl]
                r.cell_layers = int(np.sum((t - b + 1)[t > 0]))
        self.bytes_per_cell_layer = max(self.bytes_per_cell_layer or 0.0, nbytes / self._cells(members))
        self.peak_active = max(self.peak_active, len(members))
        self.core = core
        self.deck = deck
        self.repack_s.append(time.perf_counter() - t_start)

    def _step(self) -> GomError | None:
        """One step of every run in the pack; the step's error, if any."""
        self.core.step_launch()
        try:
            self.core.step_wait()
        except GomError as e:
            return e
        return None

    def tick(self, clock) -> list[Request]:
        if self.core is None:
            return []
        err = self._step()
        culprit = None
        if err is not None:
            st = err.status
            if st is not None and st.code and 0 <= st.run < len(self.members):
                culprit = st.run
            self.core.status(clear=True)
        self.elapsed += self.deck.params.dt
        now = clock()
        done = []
        for i, r in enumerate(self.members):
            if r.finished >= 0:
                continue
            r.done_steps += 1
            failed = err is not None and (culprit is None or culprit == i)
            if failed:
                r.error = str(err)
                self.failed_runs += 1
            if r.done_steps >= r.steps or failed:
                r.finished = now
                if self.on_finish:
                    self.on_finish(r, self.core, i, self.deck)
                done.append(r)
        if culprit is not None:
            self._gc_now = True
        return done


def serve_packed(lib, requests: list[Request], budget_bytes: float, precision: int = 1,
                 min_interval: float = 0.5) -> dict:
    """Replay a request stream in wall time through a PackedServer."""
    srv = PackedServer(lib, budget_bytes, precision, min_interval)
    pending = sorted(requests, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    clock = lambda: time.perf_counter() - t0  # noqa: E731
    finished = 0
    i = 0
    work = 0
    while finished < len(requests):
        now = clock()
        while i < len(pending) and pending[i].arrival <= now:
            srv.waiting.append(pending[i])
            i += 1
        srv.maybe_repack(now)
        finished += len(srv.rejected)
        srv.rejected.clear()
        live = srv.active()
        if not live:
            if i < len(pending):
                time.sleep(max(0.0, min(0.01, pending[i].arrival - now)))
            continue
        work += sum(r.cell_layers for r in live)
        finished += len(srv.tick(clock))
    srv.maybe_repack(clock())
    if srv.core is not None:
        srv.core.close()
    out = _summary(requests, clock(), work, srv.peak_bytes, srv.peak_active)
    out["repacks"] = srv.repacks
    rs = np.array(srv.repack_s) if srv.repack_s else np.zeros(1)
    out["repack_s_mean"] = float(rs.mean())
    out["repack_s_max"] = float(rs.max())
    out["repack_s_total"] = float(rs.sum())
    out["failed_runs"] = srv.failed_runs
    return out
