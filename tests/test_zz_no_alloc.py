"""The allocation-free pseudo-line compaction, qsl_cook_pseudo_line_noalloc.

It serves callers that cannot allocate device memory (their host runtime owns
the GPU's memory pool, or they only hold borrowed device pointers), so its
scratch is a fixed array inside the library instead of a caller workspace.
Called through the C ABI twice in a row, its outputs must equal those of the
workspace entry qsl_cook_pseudo_line exactly (the same kernels run on the
same inputs; the shared scratch keeps the previous call's contents, which
must not leak into the next).  This file sorts last so that a run stopping at
the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _inputs(n0, n1, nplanes, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = n0 * n1 * nplanes
    bflag = (torch.rand(n, generator=g) < 0.07).to(torch.int32)
    flags = torch.randint(1, 7, (n,), generator=g, dtype=torch.int32)
    flags[torch.rand(n, generator=g) < 0.05] = 42
    xs, ys, zs = (torch.rand(n, generator=g) * 60 for _ in range(3))
    bzi, bzo = (torch.randn(n, generator=g) for _ in range(2))
    return [t.cuda() for t in (bflag, xs, ys, zs, flags, bzi, bzo)], n


def _outputs(n):
    f = [torch.full((4 * n,), float("nan"), device="cuda") for _ in range(3)]
    b = [torch.full((n,), float("nan"), device="cuda") for _ in range(2)]
    pix = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    cnt = torch.full((2,), -1, dtype=torch.int64, device="cuda")
    return f, b, pix, cnt


def _collect(f, b, pix, cnt):
    k = int(cnt[0].item())
    return k, int(cnt[1].item()), [t[:4 * k].cpu().numpy() for t in f] + [t[:k].cpu().numpy() for t in b] + [
        pix[:k].cpu().numpy()]


def _call_workspace(lib, ins, n, n0, n1, interior, stride):
    from fastqsl_gb300.api import ptr, stream_handle
    f, b, pix, cnt = _outputs(n)
    wb = int(lib.qsl_cook_workspace_bytes(n))
    work = torch.empty((wb + 7) // 8, dtype=torch.int64, device="cuda")
    rc = lib.qsl_cook_pseudo_line(*[ptr(t) for t in ins], n, n0, n1, interior, stride,
                                  *[ptr(t) for t in f], *[ptr(t) for t in b], ptr(pix), ptr(cnt), ptr(work), wb,
                                  stream_handle())
    assert rc == 0, lib.qsl_last_error()
    torch.cuda.synchronize()
    return _collect(f, b, pix, cnt)


def _call_noalloc(lib, ins, n, n0, n1, interior, stride):
    from fastqsl_gb300.api import ptr, stream_handle
    f, b, pix, cnt = _outputs(n)
    rc = lib.qsl_cook_pseudo_line_noalloc(*[ptr(t) for t in ins], n, n0, n1, interior, stride,
                                          *[ptr(t) for t in f], *[ptr(t) for t in b], ptr(pix), ptr(cnt),
                                          stream_handle())
    assert rc == 0, lib.qsl_last_error()
    torch.cuda.synchronize()
    return _collect(f, b, pix, cnt)


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastqsl_gb300 import _build, _lib
    _build.build()
    return _lib.load()


def test_noalloc_matches_workspace_entry_twice(lib):
    # a large call then a smaller one: the second must not see the first's
    # scratch contents
    cases = [((130, 97, 5), 3, 1, 0.5), ((41, 58, 2), 4, 0, 0.25)]
    for (n0, n1, npl), seed, interior, stride in cases:
        ins, n = _inputs(n0, n1, npl, seed)
        k_ref, s_ref, ref = _call_workspace(lib, ins, n, n0, n1, interior, stride)
        k, s, got = _call_noalloc(lib, ins, n, n0, n1, interior, stride)
        assert k == k_ref and s == s_ref == 4 * k_ref
        assert k > 0
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b)


def test_noalloc_allocates_nothing(lib):
    """After a warm-up call (which looks up the scratch array's address), a
    further call leaves the device's free memory exactly as it was."""
    ins, n = _inputs(64, 80, 3, 9)
    _call_noalloc(lib, ins, n, 64, 80, 1, 0.5)
    from fastqsl_gb300.api import ptr, stream_handle
    f, b, pix, cnt = _outputs(n)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc = lib.qsl_cook_pseudo_line_noalloc(*[ptr(t) for t in ins], n, 64, 80, 1, 0.5,
                                          *[ptr(t) for t in f], *[ptr(t) for t in b], ptr(pix), ptr(cnt),
                                          stream_handle())
    assert rc == 0, lib.qsl_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert int(cnt[0].item()) > 0


def test_noalloc_rejects_oversize(lib):
    from fastqsl_gb300.api import stream_handle
    big = int(lib.qsl_cook_noalloc_max_pixels()) + 1
    dummy = torch.zeros(4, dtype=torch.int64, device="cuda")
    p = dummy.data_ptr()
    rc = lib.qsl_cook_pseudo_line_noalloc(*([p] * 7), big, 1, big, 0, 1.0, *([p] * 7), stream_handle())
    assert rc == -4
    assert b"exceed" in lib.qsl_last_error()
