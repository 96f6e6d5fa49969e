"""Regenerates tests/golden/oracle_digests.json from the CPU oracle.

Each case is a seeded synthetic scene run through the oracle: FNV-1a digests
(native/main.rs:152-163) of the moments and fields after one field solve and
of the particles after `steps` full frames.  The fixtures freeze the oracle so
the CPU tests catch any drift in it, and the GPU tests compare the CUDA path
against the same numbers.

    python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "fmm-rainbow_gb300"))

CASES = [
    # name, kind, n, seed, gravity, softening, dt, steps
    ("uniform_65536", "uniform", 65536, 1, 1.0, 1e-3, 1e-3, 1),
    ("plummer_16384", "plummer", 16384, 2, 1.0, 1e-3, 5e-4, 3),
    ("clusters_40000", "clusters", 40000, 3, 1.0, 5e-4, 5e-4, 3),
    ("uniform_4096", "uniform", 4096, 4, 1.0, 1e-3, 5e-4, 2),
    ("galaxy_65536", "galaxy", 65536, 0, 0.34, 0.012, 0.0009, 2),
]


def scene(kind, n, seed):
    from oracle import oracle as O
    from rfmm import scenes
    if kind == "galaxy":
        return O.initialize(n)
    return scenes.make(kind, n, seed)


def compute():
    from oracle import oracle as O
    out = {}
    for name, kind, n, seed, g, eps, dt, steps in CASES:
        p = scene(kind, n, seed)
        params = O.make_params(n, gravity=g, softening=eps, dt=dt)
        st = O.OracleState(p, params)
        st.solve_fields()
        entry = {"kind": kind, "n": n, "seed": seed, "gravity": g, "softening": eps, "dt": dt,
                 "steps": steps, "depth": params.depth, "scale": params.scale,
                 "input_particles": O.fnv1a(p),
                 "solve_moments": O.fnv1a(st.moments), "solve_fields": O.fnv1a(st.fields)}
        st = O.OracleState(p, params)
        st.step(steps)
        entry["step_particles"] = O.fnv1a(st.particles)
        entry["step_moments"] = O.fnv1a(st.moments)
        entry["step_fields"] = O.fnv1a(st.fields)
        out[name] = entry
    return out


if __name__ == "__main__":
    data = compute()
    with open(os.path.join(HERE, "oracle_digests.json"), "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    print(json.dumps(data, indent=1, sort_keys=True))
