"""The oracle-side generator of the benchmark's inputs (oracle/workload.py, used
by bench.py's CPU legs so that they never load the product library) gives the
same lattices and coefficients as the product's generator."""
import numpy as np


def test_workload_matches_product_generator(oracle_mod):
    from latticemontecarlo_gb300 import synthetic as S
    from oracle import workload as W

    for el, seed in ((("Al", "Mg", "Zn"), 1234), (("Al", "Cu", "Mg", "Zn"), 4321)):
        assert W.make_coefficients(el, seed) == S.make_coefficients(el, seed)
        assert W.theta_labels(el) == S.theta_labels(el)
    ns, sp, temps = S.batched_replicas(1234, 24)
    ns2, temps2 = W.batched_edges_and_temperatures(1234, 24)
    assert np.array_equal(ns, ns2) and np.array_equal(temps, temps2)
    offs = np.concatenate([[0], np.cumsum(4 * ns.astype(np.int64) ** 3)])
    for r in range(24):
        assert np.array_equal(sp[offs[r]:offs[r + 1]], W.batched_replica_lattice(1234, r, ns[r]))
    c = W.CMC_SINGLE
    assert np.array_equal(W.make_lattice(c["n"], c["fractions"], 0, 4321, c["elements"]),
                          S.make_lattice(c["n"], c["fractions"], 0, 4321, c["elements"]))
    assert W.KMC_BATCHED == S.KMC_BATCHED and W.CMC_SINGLE == S.CMC_SINGLE
