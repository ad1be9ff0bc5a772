"""nbh_diagnostics on GB300 against the FP64 restatement, and conservation over a run."""
import numpy as np
import pytest

from helpers import gpu_sim, plummer

import oracle as O

pytestmark = pytest.mark.gpu


def _check(d, r, rtol_pot=2e-6):
    assert abs(d["mass"] - r["mass"]) <= 1e-12 * r["mass"]
    np.testing.assert_allclose(d["com"], r["com"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(d["momentum"], r["momentum"], rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(d["angular_momentum"], r["angular_momentum"], rtol=1e-9, atol=1e-13)
    assert abs(d["kinetic"] - r["kinetic"]) <= 1e-10 * r["kinetic"]
    if "potential" in d:
        assert abs(d["potential"] - r["potential"]) <= rtol_pot * abs(r["potential"])
        assert abs(d["potential_unsoftened"] - r["potential_unsoftened"]) <= rtol_pot * abs(r["potential_unsoftened"])


def test_diagnostics_match_fp64_single_universe():
    n = 5000
    arrs = plummer(n, seed=31)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    g.load(*arrs)
    g.step(2)
    st = g.read()
    (d,) = g.diagnostics(potential=True)
    r = O.diagnostics_f64(st["x"], st["y"], st["z"], st["vx"], st["vy"], st["vz"], arrs[6], eps=0.05)
    _check(d, r)
    assert d["max_depth"] == g.stats()["max_depth"]
    assert abs(d["total"] - (r["kinetic"] + r["potential"])) <= 2e-6 * abs(r["potential"])
    # a Plummer sphere drawn from its distribution function is in virial equilibrium
    assert abs(2 * d["kinetic"] / d["potential"] + 1) < 0.1


def test_diagnostics_per_universe_of_a_batch():
    from nbh import universe as U
    counts = [700, 1, 3000, 257]
    parts = [U.PlummerUniverseGenerator(seed=70 + i).arrays(c) for i, c in enumerate(counts)]
    cat = [np.concatenate([p[k] for p in parts]) for k in range(7)]
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    g.load_batch(counts, *cat)
    g.step(1)
    st = g.read()
    ds = g.diagnostics(potential=True)
    assert len(ds) == len(counts)
    off = 0
    for d, c, p in zip(ds, counts, parts):
        sl = slice(off, off + c)
        r = O.diagnostics_f64(st["x"][sl], st["y"][sl], st["z"][sl], st["vx"][sl], st["vy"][sl], st["vz"][sl],
                              p[6], eps=0.05)
        _check(d, r)
        off += c
    # moments only: the potential fields are absent
    assert "potential" not in g.diagnostics()[0]


def test_reference_energy_form_is_twice_the_unsoftened_potential():
    n = 512
    arrs = plummer(n, seed=32)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    g.load(*arrs)
    (d,) = g.diagnostics(potential=True)
    ref = O.reference_energy(*arrs)
    assert abs(ref["epot"] + 2 * d["potential_unsoftened"]) <= 2e-6 * ref["epot"]
    assert abs(ref["ekin"] - d["kinetic"]) <= 1e-10 * ref["ekin"]


def test_energy_and_momentum_conserved_over_a_run():
    """32,768-body Plummer sphere, theta 0.5, eps 0.05, dt 0.005, 200 steps (one time unit):
    total energy (softened potential) and momentum drift stay small."""
    n = 32768
    arrs = plummer(n, seed=33)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.005)
    g.load(*arrs)
    g.step(1)
    (d0,) = g.diagnostics(potential=True)
    g.step(200)
    (d1,) = g.diagnostics(potential=True)
    de = abs(d1["total"] - d0["total"]) / abs(d0["total"])
    dp = np.linalg.norm(np.subtract(d1["momentum"], d0["momentum"]))
    dl = np.linalg.norm(np.subtract(d1["angular_momentum"], d0["angular_momentum"]))
    print("energy drift %.2e, momentum drift %.2e, angular momentum drift %.2e" % (de, dp, dl))
    assert de < 1e-4
    assert dp < 1e-4
    assert dl < 1e-4
