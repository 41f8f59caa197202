"""Batched persistent counting (one launch, CUDA-graph replay) against the
per-graph launch path and the oracle."""
import numpy as np
import pytest

import oracle
from trianglecount_gb300 import generators as gen

pytestmark = pytest.mark.gpu


def test_uneven_batch_matches_per_graph_and_oracle(ctx):
    specs = gen.batch_mix(48, scale=0.05)
    graphs, want = [], []
    for s in specs:
        src, dst = s.edges()
        orp, ocl, t = oracle.pipeline(src, dst)
        graphs.append(ctx.upload(orp, ocl))
        want.append(t)
    b = ctx.batch(graphs)
    for _ in range(3):  # graph replays give the same answer
        assert list(b.run()) == want
    assert list(ctx.count_each(graphs)) == want


def test_batch_async_and_single(ctx):
    src, dst = gen.rmat(13)
    orp, ocl, t = oracle.pipeline(src, dst)
    g = ctx.upload(orp, ocl)
    b = ctx.batch([g])
    b.run_async()
    assert list(b.results()) == [t]
    # the same graph several times in one batch
    assert list(ctx.batch([g, g, g]).run()) == [t, t, t]
