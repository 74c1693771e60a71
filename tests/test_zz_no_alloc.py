"""The allocation-free transform entry point (pg_nm_transform_noalloc).

Some callers cannot call cudaMalloc: a Fortran / MPI host program that gives
all of the GPU's memory to its own pool at start-up, or code in a section where
cudaMalloc's implicit device synchronisation is not allowed.  This entry point
uses only a static device array for its scratch.  The test calls it through the
C-ABI on caller-owned device buffers, twice in a row (the scratch keeps the
previous call's contents), and compares each result with the allocating entry
point pg_nm_transform(PG_MIXED) within the split-BF16 tolerance the other
transform tests use.  It lives in its own file so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_transform_matches_allocating_entry_point(pg, ctx):
    torch = pytest.importorskip("torch")
    P = 128
    for call, ncol in enumerate((300, 77)):
        cols = np.random.RandomState(11 + call).randn(ncol, P)
        ref = ctx.nm_transform(P, cols.ravel(), pg.PG_MIXED).reshape(ncol, P)
        d_in = torch.from_numpy(cols.copy()).cuda()
        d_out = torch.full_like(d_in, float("nan"))
        torch.cuda.synchronize()
        rc = pg.lib().pg_nm_transform_noalloc(P, ncol, C.c_void_p(d_in.data_ptr()),
                                              C.c_void_p(d_out.data_ptr()), None)
        pg.check(rc)
        out = d_out.cpu().numpy()
        assert np.all(np.isfinite(out))
        assert np.max(np.abs(out - ref)) <= 3e-5 * np.max(np.abs(ref))


def test_noalloc_transform_rejects_sizes_beyond_its_scratch(pg):
    rc = pg.lib().pg_nm_transform_noalloc(256, 4, C.c_void_p(1), C.c_void_p(1), None)
    assert rc == pg.PG_ERR_ARG
    assert "P must be 128" in pg.lib().pg_last_error().decode()
