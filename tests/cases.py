"""Shared problem builders for the tests: the configurations' PDEs, element tables and
seeded inputs, built with the product's own host code (asgkron.pdes / asgkron.grid)."""
import numpy as np

import asgkron
from asgkron import pdes


def problem(name, lev, deg, LF=-1.0, max_lev=8):
    """(pde, table, idx1d[N,d] 1-based, term_mats) for one of the configuration PDEs."""
    if name == "continuity2":
        pde = pdes.continuity2(lev, LF)
    elif name == "continuity3":
        pde = pdes.continuity3(lev, LF)
    elif name == "continuity6":
        pde = pdes.continuity6(lev, LF)
        max_lev = 4
    elif name == "diffusion2":
        pde = pdes.diffusion2(lev)
    else:
        raise KeyError(name)
    table = asgkron.hash_table_sparse_nD(pde.levels, max(max_lev, max(pde.levels)))
    idx = table.idx1d()
    mats = pde.term_mats(deg)
    return pde, table, idx, mats


def random_problem(seed, d, lev, deg):
    """Dense random N(0, 1/deg) operators on an SG table (the batched configuration's model)."""
    rng = np.random.default_rng(seed)
    table = asgkron.hash_table_sparse_nD([lev] * d, max(8, lev))
    idx = table.idx1d()
    n = deg * 2 ** lev
    mats = [[rng.normal(0.0, 1.0 / np.sqrt(deg), (n, n)) for _ in range(d)] for _ in range(d)]
    return table, idx, mats


def rel2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
