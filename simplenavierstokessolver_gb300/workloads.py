"""Seeded synthetic workloads: the 64-case ensemble and the serving stream.

Every random draw comes from SplitMix64 (Steele, Lea and Flood, 2014) seeded
per case with s0 + k (s0 = 20261203), so a case is reproducible on its own:
  ensemble case k: nx uniform in {64, 128, 256}, ny = 2 nx, lx = 1, ly = 2,
    log10 Ra uniform in [6, 9], Pr uniform in [0.7, 7], temperature noise
    uniform in [-0.05, 0.05] from the same seed (sns_case_desc.seed);
  serving request k: nx uniform in {64, 128, 256, 512}, ny = 2 nx,
    log10 Ra uniform in [6, 10], Pr uniform in [0.7, 7], steps uniform in
    {200, ..., 2000}; arrivals form a Poisson process of the given rate
    (exponential gaps from SplitMix64(s0 - 1)).
"""
from __future__ import annotations

import math

from .batch import Desc

S0 = 20261203
MASK = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & MASK

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)

    def choice(self, items):
        return items[self.next() % len(items)]


def ensemble(n: int = 64, s0: int = S0, steps: int = 0) -> list[Desc]:
    out = []
    for k in range(n):
        g = SplitMix64(s0 + k)
        nx = g.choice([64, 128, 256])
        ra = 10.0 ** (6.0 + 3.0 * g.uniform())
        pr = 0.7 + 6.3 * g.uniform()
        out.append(Desc(nx, 2 * nx, ly=2.0, Ra=ra, Pr=pr, seed=s0 + k, steps=steps))
    return out


def serving_stream(rate_per_s: float, duration_s: float, s0: int = S0,
                   nx_choices=(64, 128, 256, 512), steps_range=(200, 2000)):
    """requests (Desc with steps) and their arrival times in seconds"""
    gaps = SplitMix64(s0 - 1)
    t, descs, arrivals, k = 0.0, [], [], 0
    while True:
        t += -math.log(1.0 - gaps.uniform()) / rate_per_s
        if t > duration_s:
            break
        g = SplitMix64(s0 + 1000 + k)
        nx = g.choice(list(nx_choices))
        ra = 10.0 ** (6.0 + 4.0 * g.uniform())
        pr = 0.7 + 6.3 * g.uniform()
        steps = steps_range[0] + g.next() % (steps_range[1] - steps_range[0] + 1)
        descs.append(Desc(nx, 2 * nx, ly=2.0, Ra=ra, Pr=pr, seed=s0 + 1000 + k, steps=steps))
        arrivals.append(t)
        k += 1
    return descs, arrivals
