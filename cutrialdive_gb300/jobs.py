"""Heterogeneous trial-factoring job mixes (the batched and served workloads).

A job mix is drawn from a seeded generator in a fixed draw order
(family -> parameter -> length -> start -> a):

* family uniform over {smarandache, riesel, proth_fixed_n, mersenne};
* parameter: smarandache base b uniform in 2..16, riesel k odd uniform in
  [3, 999999], proth_fixed_n n uniform in [1000, 20000], mersenne none;
* index range [start, start + len) with len = round(exp(U(ln 100, ln 20000)))
  and start uniform in [1, 50000];
* prime range [2^a, 2^(a+2)) with a uniform in {30, ..., 38}.

Serving mixes add Poisson arrival times (exponential gaps at a given rate)
drawn from the same generator after the jobs.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import asdict, dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FAMILIES = ["smarandache", "riesel", "proth_fixed_n", "mersenne"]
FAMILY_IDS = {"smarandache": 3, "riesel": 2, "proth_fixed_n": 6, "mersenne": 0}


@dataclass
class Job:
    family: str
    param: int
    n0: int
    n1: int
    a: int

    @property
    def f0(self) -> int:
        return 1 << self.a

    @property
    def f1(self) -> int:
        return 1 << (self.a + 2)

    def ctd(self, max_factors: int = 32, shrink: int = 1):
        """The job as a ctd_job; shrink > 1 keeps the first 1/shrink of its
        prime range, [2^a, 2^a + 3 * 2^a / shrink) (a bounded sample)."""
        from ._native import CtdJob

        f1 = self.f0 + (self.f1 - self.f0) // shrink
        return CtdJob(FAMILY_IDS[self.family], max_factors, self.param, self.n0, self.n1, self.f0, f1)


def draw_jobs(seed: int, count: int) -> tuple[list[Job], np.random.Generator]:
    rng = np.random.default_rng(seed)
    jobs = []
    for _ in range(count):
        fam = FAMILIES[int(rng.integers(0, 4))]
        if fam == "smarandache":
            param = int(rng.integers(2, 17))
        elif fam == "riesel":
            param = 2 * int(rng.integers(1, 500000)) + 1
        elif fam == "proth_fixed_n":
            param = int(rng.integers(1000, 20001))
        else:
            param = 0
        length = int(round(math.exp(rng.uniform(math.log(100), math.log(20000)))))
        start = int(rng.integers(1, 50001))
        a = int(rng.integers(30, 39))
        jobs.append(Job(fam, param, start, start + length, a))
    return jobs, rng


def batched_mix() -> list[Job]:
    """64 jobs from seed 1234 (the batched configuration)."""
    return draw_jobs(1234, 64)[0]


def served_mix(rate: float, count: int = 2000, seed: int = 99) -> tuple[list[Job], list[float]]:
    """2000 jobs from seed 99 with Poisson arrival times at `rate` jobs/s."""
    jobs, rng = draw_jobs(seed, count)
    gaps = rng.exponential(1.0 / rate, size=count)
    return jobs, list(np.cumsum(gaps))


# prime counts pi(2^k) (k = 30..40), for work estimates
PI_POW2 = {30: 54400028, 31: 105097565, 32: 203280221, 33: 393615806, 34: 762939111, 35: 1480206279,
           36: 2874398515, 37: 5586502348, 38: 10866266172, 39: 21151907950, 40: 41203088796}


def updates(job: Job) -> int:
    """Residue updates of a job: primes in [2^a, 2^(a+2)) x terms."""
    return (PI_POW2[job.a + 2] - PI_POW2[job.a]) * (job.n1 - job.n0)


def write_mix(path: str, jobs: list[Job]) -> None:
    with open(path, "w") as fh:
        json.dump([asdict(j) for j in jobs], fh, indent=0)


if __name__ == "__main__":
    mix = batched_mix()
    write_mix(os.path.join(HERE, "jobs_batched_seed1234.json"), mix)
    total = sum(updates(j) for j in mix)
    print(f"64 jobs, {total:.4e} updates")
