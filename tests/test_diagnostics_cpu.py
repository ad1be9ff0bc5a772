"""The FP64 diagnostics restatement against the reference's printEnergy / printImpulse
formulas (GPUBarnesHutNBodySimulation.java:305-365), on the CPU."""
import numpy as np

import oracle as O


def _universe(n, seed):
    r = np.random.default_rng(seed)
    x, y, z = r.uniform(-1, 1, (3, n))
    vx, vy, vz = r.normal(0, 0.1, (3, n))
    m = r.uniform(0.5, 1.5, n) / n
    return x, y, z, vx, vy, vz, m


def test_reference_epot_counts_each_pair_twice():
    arrs = _universe(200, 3)
    ref = O.reference_energy(*arrs)
    d = O.diagnostics_f64(*arrs, eps=0.05)
    assert abs(ref["ekin"] - d["kinetic"]) <= 1e-13 * abs(ref["ekin"])
    # the reference's epot is positive and doubled: epot = -2 * (sum over pairs once)
    assert abs(ref["epot"] + 2 * d["potential_unsoftened"]) <= 1e-12 * abs(ref["epot"])
    assert abs(ref["etot"] - (d["kinetic"] + 2 * d["potential_unsoftened"])) <= 1e-12 * abs(ref["epot"])


def test_momentum_and_centre_of_mass():
    x, y, z, vx, vy, vz, m = _universe(300, 4)
    d = O.diagnostics_f64(x, y, z, vx, vy, vz, m, eps=0.05, potential=False)
    np.testing.assert_allclose(d["momentum"], [(m * vx).sum(), (m * vy).sum(), (m * vz).sum()], rtol=1e-13)
    np.testing.assert_allclose(d["com"], [(m * x).sum() / m.sum(), (m * y).sum() / m.sum(), (m * z).sum() / m.sum()],
                               rtol=1e-13)
    L = np.cross(np.stack([x, y, z], 1), np.stack([vx, vy, vz], 1)) * m[:, None]
    np.testing.assert_allclose(d["angular_momentum"], L.sum(0), rtol=1e-12, atol=1e-15)


def test_softened_potential_two_bodies():
    """Two unit masses at distance 1, eps 0.5: -1/sqrt(1.25) softened, -1 unsoftened."""
    x = np.array([0.0, 1.0]); z0 = np.zeros(2); m = np.ones(2)
    d = O.diagnostics_f64(x, z0, z0, z0, z0, z0, m, eps=0.5)
    assert abs(d["potential"] + 1 / np.sqrt(1.25)) < 1e-12
    assert abs(d["potential_unsoftened"] + 1.0) < 1e-12
