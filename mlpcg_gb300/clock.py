"""Nested wall-clock timers with the interface of the reference's GlobalClock
(lib/global_clock.py:19-52): ``start(name)`` / ``stop(name)`` nest, ``report()``
prints, ``top_level_clocks['Total'].tot_time`` is read by test.py."""
from __future__ import annotations

import time


class SingleClock:
    def __init__(self, name, indent=0):
        self.name = name
        self.indent = indent
        self.tot_time = 0.0
        self.children = {}
        self.start = 0.0

    def start_timer(self):
        self.start = time.perf_counter()

    def stop_timer(self):
        self.tot_time += time.perf_counter() - self.start

    def info(self):
        s = "  " * self.indent + self.name + ": " + str(self.tot_time) + "\n"
        for c in self.children.values():
            s += c.info()
        return s


class GlobalClock:
    def __init__(self):
        self.top_level_clocks = {}
        self.scope = []

    def start(self, name):
        if not self.scope:
            clock = self.top_level_clocks.setdefault(name, SingleClock(name))
        else:
            parent = self.scope[-1]
            clock = parent.children.setdefault(name, SingleClock(name, indent=len(self.scope)))
        clock.start_timer()
        self.scope.append(clock)

    def stop(self, name):
        if not self.scope:
            raise Exception(f"Clock '{name}' was not initialized.")
        if name != self.scope[-1].name:
            raise Exception("Timers must be stopped in order.")
        self.scope.pop().stop_timer()

    def report(self):
        for clock in self.top_level_clocks.values():
            print(clock.info())
