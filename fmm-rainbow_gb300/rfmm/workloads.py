"""The measured workloads: seeded synthetic scenes with the shapes, sizes and
value distributions of the five solver configurations.

Shared by the bench and by the parity tests that run the benchmarked
configurations in full, so both see the same bytes.

  * uniform_64k  -- 65,536 bodies uniform in [0,1)^3, zero velocities,
                    one force evaluation + one leapfrog step at dt 1e-3;
  * plummer_1m   -- the default preset size, 1,048,576 bodies, Plummer sphere
                    a = 0.1 at the box centre truncated at r = 0.5, 60 steps
                    at dt 5e-4 (the headline configuration);
  * clusters_5m  -- the budget maximum, 5,242,880 bodies in 8 Plummer
                    clusters, eps 5e-4, 60 steps;
  * batched_256  -- 256 scenes of N log-uniform in [4096, 262144], half
                    uniform cube, half Plummer, 60 steps per bench step;
  * served       -- Poisson request arrivals, N log-uniform in
                    [16384, 2097152] (uniform / Plummer / 4-cluster), steps
                    uniform in [1, 60], 150 GB device-memory budget.
"""
from __future__ import annotations

import numpy as np

from . import PARTICLE_DTYPE, scenes

WORKLOADS = {
    "plummer_1m": dict(kind="plummer", n=1 << 20, seed=2, fmm_steps=60, dt=5e-4, eps=1e-3, G=1.0,
                       desc="Plummer sphere a=0.1 at (0.5,0.5,0.5), r<0.5, N=1,048,576, "
                            "G=1, eps=1e-3, 60 steps dt=5e-4, Plummer-DF velocities"),
    "uniform_64k": dict(kind="uniform", n=65536, seed=1, fmm_steps=1, dt=1e-3, eps=1e-3, G=1.0,
                        desc="uniform [0,1)^3, N=65,536, G=1, eps=1e-3, v=0, 1 step dt=1e-3"),
    "clusters_5m": dict(kind="clusters", n=5242880, seed=3, fmm_steps=60, dt=5e-4, eps=5e-4, G=1.0,
                        desc="8 Plummer clusters a~logU[0.02,0.1], centres U[0.2,0.8]^3, "
                             "N=5,242,880, eps=5e-4, bulk sigma 0.05, 60 steps dt=5e-4"),
    "served": dict(kind="served", n_min=16384, n_max=2097152, steps_max=60, seed=5, dt=5e-4,
                   eps=1e-3, G=1.0, rates=[50, 200, 500, 1000, 2000], requests=10000,
                   budget=150 << 30, fmm_steps=None,
                   desc="requests with N log-uniform [16384, 2097152] (uniform / Plummer / "
                        "4-cluster), steps U[1,60], dt=5e-4, eps=1e-3, Poisson arrivals"),
    "batched_256": dict(kind="batched", scenes=256, n_min=4096, n_max=262144, seed=4,
                        fmm_steps=60, dt=5e-4, eps=1e-3, G=1.0,
                        desc="256 scenes, N log-uniform [4096, 262144], half uniform cube, "
                             "half Plummer a=0.1, G=1, eps=1e-3, 60 steps dt=5e-4"),
}


def scene(w) -> np.ndarray:
    """The single scene of a plain workload."""
    return scenes.make(w["kind"], w["n"], w["seed"])


def batch_scenes(w):
    """The batched workload's scenes: seeded sizes, alternating uniform / Plummer."""
    rng = np.random.default_rng(w["seed"])
    sizes = np.exp(rng.uniform(np.log(w["n_min"]), np.log(w["n_max"]), w["scenes"])).astype(int)
    return [scenes.make("uniform" if i % 2 == 0 else "plummer", int(n), 1000 + i)
            for i, n in enumerate(sizes)]


SERVED_KINDS = ("uniform", "plummer", "clusters4")


class RequestPool:
    """The served workload's requests without one scene generation per request.

    One seeded parent sample of n_max bodies is drawn per scene kind; request
    i takes `n_i` consecutive bodies of its kind's parent starting at a seeded
    offset.  The parent's bodies are independent draws from the kind's
    distribution in a random order (the cluster mixture is shuffled, the
    uniform and Plummer samples are i.i.d.), so every request is itself a
    seeded sample of that distribution with n_i bodies; masses are 1/n_i
    (the solver takes them from the body count).
    """

    def __init__(self, w, count: int):
        rng = np.random.default_rng(w["seed"])
        self.n = np.exp(rng.uniform(np.log(w["n_min"]), np.log(w["n_max"]), count)).astype(np.int64)
        self.steps = rng.integers(1, w["steps_max"] + 1, count)
        self.kind = np.arange(count) % len(SERVED_KINDS)
        self.parents = [scenes.make(k, int(w["n_max"]), 7000 + j)
                        for j, k in enumerate(SERVED_KINDS)]
        span = int(w["n_max"]) - self.n
        self.offset = (rng.random(count) * (span + 1)).astype(np.int64)

    def __len__(self):
        return len(self.n)

    def bodies(self, i: int) -> np.ndarray:
        """Request i's bodies: a contiguous view (no copy) of its kind's parent."""
        p = self.parents[int(self.kind[i])]
        o = int(self.offset[i])
        return p[o: o + int(self.n[i])]

    def body_steps(self) -> int:
        return int(np.sum(self.n * self.steps))


def served_pool(w, count: int) -> RequestPool:
    return RequestPool(w, count)


def roofline_bytes_integrate(n, cells, depth):
    """Algorithmic bytes of one fused integrate launch.

    64 B per body (32 B particle in, 32 B out), 64 B per tree cell (48 B field
    + 16 B moment gathered once) and 16 B per leaf cell (the next step's leaf
    deposit written once).
    """
    return 64 * n + 64 * cells + 16 * 8 ** depth


assert PARTICLE_DTYPE.itemsize == 32
