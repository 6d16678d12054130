"""The allocation-free PageRank step (grz_pr_step_noalloc) against the regular entry point.

Some callers cannot allocate device memory while they run.  Their framework's own pool may
own it, cudaMalloc may be too costly inside a latency-bound loop, or allocation may be
forbidden after start-up.  For them the library offers one PageRank iteration whose scratch
is a fixed device array inside the library.  This test calls it through the C ABI, twice in a
row (the second call reads the first call's output), and checks each result against the
regular entry point, grz_pr_iterate.  The tolerance is the PageRank tolerance of the other
tests: 1e-12 relative L1.  The file name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
PR_TOL = 1e-12


def test_noalloc_step_matches_pr_iterate_twice():
    import torch

    from grazelle import graphgen as gg, native
    from grazelle.engine import Graph

    g = gg.rmat(16, seed=11)
    V = g.num_vertices
    with Graph(0) as G:
        G.load_pairs(V, g.pull_order().pairs(), g.push_order().pairs())
        info = G.info()
        expected = []
        for iters in (1, 2):
            expected.append(G.pagerank(iters, damping=0.875))
        p0 = G.pr_init(0.875).props()             # initial props (rank / outdeg')
        od = G.outdegrees()
        lib = G.lib
        assert lib.grz_pr_step_noalloc_max_vertices() == 1 << 18
        # caller-owned device arrays: allocated here by the caller, never by the entry point
        dev_in = torch.from_numpy(p0).cuda()
        dev_od = torch.from_numpy(od).cuda()
        dev_out = torch.empty_like(dev_in)
        torch.cuda.synchronize()
        for step in range(2):
            rc = lib.grz_pr_step_noalloc(C.c_void_p(info.pull_list_device), info.pull_vectors, V,
                                         C.c_void_p(dev_in.data_ptr()), C.c_void_p(dev_od.data_ptr()), C.c_double(0.875),
                                         C.c_void_p(dev_out.data_ptr()), None)
            assert rc == native.GRZ_OK
            torch.cuda.synchronize()
            got = dev_out.cpu().numpy()
            assert O.relative_l1(got, expected[step]) < PR_TOL, step
            dev_in, dev_out = dev_out, dev_in


def test_noalloc_step_rejects_oversized_graphs():
    from grazelle import native
    lib = native.load()
    too_big = (1 << 18) + 1
    rc = lib.grz_pr_step_noalloc(C.c_void_p(32), 1, too_big, C.c_void_p(8), C.c_void_p(8), C.c_double(0.875),
                                 C.c_void_p(8), None)
    assert rc == -5  # GRZ_ERR_RANGE, before any device work
    assert lib.grz_pr_step_noalloc(C.c_void_p(32), 1, 0, C.c_void_p(8), C.c_void_p(8), C.c_double(0.875),
                                   C.c_void_p(8), None) == -5


def test_noalloc_step_rejects_overlapping_props():
    """props_out is written while other blocks still read props_in, so overlapping ranges are
    refused with GRZ_ERR_ARG before any device work (the pointers are never dereferenced)."""
    from grazelle import native
    lib = native.load()
    V = 64
    for base_in, base_out in ((4096, 4096), (4096, 4096 + 8 * (V - 1)), (4096 + 8, 4096)):
        rc = lib.grz_pr_step_noalloc(C.c_void_p(32), 1, V, C.c_void_p(base_in), C.c_void_p(8), C.c_double(0.875),
                                     C.c_void_p(base_out), None)
        assert rc == native.GRZ_ERR_ARG, (base_in, base_out)
