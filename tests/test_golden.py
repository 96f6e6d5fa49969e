"""The oracle reproduces its frozen digests (tests/golden/oracle_digests.json,
written by tests/golden/make_golden.py): a regression pin on the checker."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "oracle_digests.json")))


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_oracle_reproduces_golden_digests(oracle_mod, name):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden
    O = oracle_mod
    g = GOLDEN[name]
    p = make_golden.scene(g["kind"], g["n"], g["seed"])
    if O.fnv1a(p) != g["input_particles"]:
        pytest.skip("this platform's scene generator differs in the last bits (libm)")
    params = O.make_params(g["n"], gravity=g["gravity"], softening=g["softening"], dt=g["dt"])
    assert params.depth == g["depth"] and params.scale == g["scale"]
    st = O.OracleState(p, params)
    st.solve_fields()
    assert O.fnv1a(st.moments) == g["solve_moments"]
    assert O.fnv1a(st.fields) == g["solve_fields"]
    st = O.OracleState(p, params)
    st.step(g["steps"])
    assert O.fnv1a(st.particles) == g["step_particles"]
    assert O.fnv1a(st.moments) == g["step_moments"]
    assert O.fnv1a(st.fields) == g["step_fields"]
