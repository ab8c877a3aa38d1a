"""Host-side checks of the backward_euler / bdf2 device fast path: which mass matrices count as
lumped and which closures are an ElasticPotential's (no GPU needed)."""

import numpy as np
import pytest
import scipy.sparse as sps

api = pytest.importorskip("simkit_gb300.api")


def test_vertex_masses_accepts_only_lumped_equal_per_vertex():
    m = np.array([1.0, 2.0, 3.0])
    M = sps.diags(np.repeat(m, 3)).tocsc()
    assert np.array_equal(api._vertex_masses(M, 3), m)
    assert np.array_equal(api._vertex_masses(M.toarray(), 3), m)
    bad = M.tolil()
    bad[0, 1] = 0.5                          # not diagonal
    assert api._vertex_masses(bad.tocsc(), 3) is None
    d = np.repeat(m, 3)
    d[1] += 1.0                              # components of one vertex differ
    assert api._vertex_masses(sps.diags(d), 3) is None
    assert api._vertex_masses(M, 4) is None  # wrong size
    assert np.array_equal(api._vertex_masses(sps.diags(np.repeat(m, 3)), 3), m)   # dia format as built


def test_potential_of_recognises_only_bound_methods_of_one_potential():
    a = object.__new__(api.ElasticPotential)
    b = object.__new__(api.ElasticPotential)
    assert api._potential_of(a.energy, a.gradient, a.hessian) is a
    assert api._potential_of(a.energy, b.gradient, a.hessian) is None          # two potentials
    assert api._potential_of(lambda x: a.energy(x), a.gradient, a.hessian) is None
    assert api._potential_of(a.gradient, a.energy, a.hessian) is None          # roles swapped
