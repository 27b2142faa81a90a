"""The CPU oracle reproduces every golden value of the reference's own unit tests
(openmp_solver/tests/test_{diffusion,bulk,dirichlet,cell}_solver.cpp)."""
import pytest

import golden_checks as G


@pytest.mark.parametrize("name,fn", G.ALL, ids=[n for n, _ in G.ALL])
def test_oracle_matches_reference_golden(oracle_mod, name, fn):
    fn(lambda: oracle_mod.OracleSolver(threads=2))
