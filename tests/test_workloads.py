"""The seeded workload generators (CPU): the parameter sweep and the serving
mix are reproducible from their seeds and draw inside the ranges their
specifications give, and their request descriptors are well formed."""
import math

import numpy as np

from nrgplusplus_gb300 import workloads


def test_sweep_is_seeded_and_in_range():
    a = workloads.sweep_instances()
    b = workloads.sweep_instances()
    assert len(a) == 512 and a == b
    assert workloads.sweep_instances(seed=workloads.SWEEP_SEED + 1) != a
    for p in a:
        assert 0.05 <= p["U"] <= 1.0
        assert abs(p["eps"] + 0.5 * p["U"]) <= 0.1
        assert 0.03 <= p["V"] <= 0.3
        assert p["lam"] in (2.0, 2.5, 3.0)
        assert p["nkeep"] in (256, 512, 1024, 2048)
        assert 30 <= p["nsites"] <= 60
    # every value of the discrete draws occurs, and V is spread in log
    assert {p["lam"] for p in a} == {2.0, 2.5, 3.0}
    assert {p["nkeep"] for p in a} == {256, 512, 1024, 2048}
    assert {p["nsites"] for p in a} >= {30, 60}
    lv = np.log([p["V"] for p in a])
    assert abs(lv.mean() - 0.5 * (math.log(0.03) + math.log(0.3))) < 0.15


def test_serving_mix_families_and_ranges():
    mix = workloads.serving_mix(2000)
    assert mix == workloads.serving_mix(2000)
    kinds = [p["kind"] for p in mix]
    frac = {k: kinds.count(k) / len(kinds) for k in ("siam", "kondo", "twochannel")}
    assert abs(frac["siam"] - 0.60) < 0.04
    assert abs(frac["kondo"] - 0.25) < 0.04
    assert abs(frac["twochannel"] - 0.15) < 0.03
    for p in mix:
        assert 30 <= p["nsites"] <= 50
        if p["kind"] == "siam":
            assert 0.05 <= p["U"] <= 1.0 and abs(p["eps"] + 0.5 * p["U"]) <= 0.1
            assert 0.03 <= p["V"] <= 0.3 and p["lam"] in (2.0, 2.5, 3.0)
            assert p["nkeep"] in (256, 512, 1024, 2048, 4096)
        elif p["kind"] == "kondo":
            assert 0.05 <= p["J"] <= 0.3 and p["lam"] == 2.5
            assert p["nkeep"] in (256, 512, 1024, 2048, 4096)
        else:
            assert 0.08 <= p["V"] <= 0.15 and p["lam"] == 4.0
            assert (p["eps"], p["U"]) == (-0.3, 0.6)
            assert p["nkeep"] in (256, 512, 1024)


def test_mix_requests_are_well_formed():
    """Hoppings and rescale factors per site in the reference drivers' forms:
    SIAM and two-channel start with the V site (rescale 1, then 1 at the
    first Wilson site and sqrt(Lambda) after), Kondo has no V site and
    rescales by sqrt(Lambda) from the first site; one hopping per f-dagger
    operator (four for the two-channel impurity)."""
    for p in workloads.serving_mix(60):
        r = workloads.mix_request(p)
        t, rs = r["t"], r["rescale"]
        nops = len(r["impurity"].fdag)
        assert t.shape[1] == nops and rs.shape == (t.shape[0],)
        assert r["nkeep"] == p["nkeep"] and r["keep_eigenvalues"]
        s = math.sqrt(p["lam"])
        if p["kind"] == "kondo":
            assert t.shape[0] == p["nsites"] and np.allclose(rs, s)
        else:
            assert t.shape[0] == p["nsites"] + 1
            assert np.allclose(t[0], p["V"]) and rs[0] == 1.0 and rs[1] == 1.0 and np.allclose(rs[2:], s)
            if p["kind"] == "twochannel":
                assert nops == 4
