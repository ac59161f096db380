"""The oracle's own workload generator (oracle/oracle_gen.c) reproduces the
product's generator bit for bit, so the CPU implementation timed beside the
GPU and the parity checks see the same seeded graphs, weights, priorities
and sources without loading a library of the product."""
import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import graphgen as gg


@pytest.mark.parametrize("V,ef,seed", [(2, 1, 1), (1000, 5, 3), (4096, 16, 1), (3000, 8.5, 2),
                                       (1 << 16, 16, 7), (50_000, 32, 11)])
def test_rmat_and_inputs_match(V, ef, seed):
    a = gg.rmat(V, ef, seed=seed)
    b = oracle.gen_rmat(V, ef, seed=seed)
    assert np.array_equal(a.row_ptr, b.row_ptr)
    assert np.array_equal(a.col, b.col)
    assert np.array_equal(gg.uniform_weights(a, 1, 255, seed=1),
                          oracle.gen_uniform_weights(b, 1, 255, seed=1))
    assert np.array_equal(gg.unique_weights(a, seed=3), oracle.gen_unique_weights(b, seed=3))
    assert np.array_equal(gg.priorities(V, seed=4), oracle.gen_priorities(V, seed=4))
    assert np.array_equal(gg.sources(a, 16, seed=2), oracle.gen_sources(b, 16, seed=2))


def test_other_quadrant_probabilities():
    a = gg.rmat(5000, 12, a=0.45, b=0.15, c=0.15, seed=9)
    b = oracle.gen_rmat(5000, 12, a=0.45, b=0.15, c=0.15, seed=9)
    assert np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col, b.col)


def test_permutation_edge_sizes():
    for n in (0, 1, 2, 17):
        assert np.array_equal(gg.permutation(n, seed=5), oracle.gen_permutation(n, seed=5))
