"""Replica of GOM's time loop (main.f90:53-304) over the C ABI.

The Fortran driver keeps its own time bookkeeping and forcing (setup_spinup, wind, boundary
elevation and discharge) and calls the per-timestep core; this module does the same through a
``GomCore`` context so that tests and benchmarks exercise the ABI the way GOM would.
"""
from __future__ import annotations

from .core import GomCore, TIME_LOOP, prepare
from .deck import Deck, HostForcing, initial_state


class Run:
    def __init__(self, deck: Deck, core: GomCore, state: dict | None = None):
        self.deck = deck
        self.core = core
        self.forcing = HostForcing(deck)
        self.it = 0
        self.pcg_iters: list[int] = []
        prepare(core, state if state is not None else initial_state(deck))

    def step(self, fused: bool = True) -> int:
        """One timestep: host forcing, then the core (fused, or one ABI call per subroutine)."""
        self.it += 1
        self.core.set_forcing(self.forcing.step(self.it))
        if fused:
            iters = self.core.step_all()
        else:
            iters = 0
            for name in TIME_LOOP:
                r = self.core.step(name)
                if name == "free_surface":
                    iters = r
        self.pcg_iters.append(iters)
        return iters

    def advance(self, n: int, fused: bool = True):
        for _ in range(n):
            self.step(fused)
