"""nsg_imfill_holes_u8_noalloc: hole filling for callers that cannot allocate
device memory.  It is checked against nsg_imfill_holes_u8 (the context-based
entry point) through the C ABI, on consecutive calls that share the library's
static work array.  This file is collected last so that the test also runs
after every other test has used the device; it passes when run on its own as
well."""
import ctypes as C

import numpy as np
import pytest

MAX_PIXELS = 4194304  # NSG_NOALLOC_MAX_PIXELS in include/nsg.h


def _mask(rows, cols, seed, p):
    rng = np.random.default_rng(seed)
    return ((rng.random((rows, cols)) < p) * 255).astype(np.uint8)


def test_noalloc_rejects_bad_arguments_without_a_device(nsg):
    from nscale_gb300 import _lib
    fake = C.c_void_p(256)  # never dereferenced: every case below is rejected first
    f = nsg.nsg_imfill_holes_u8_noalloc
    assert f(fake, fake, 2048, 2049, 4, None) == _lib.ERR_OOM
    assert f(fake, fake, MAX_PIXELS + 1, 1, 8, None) == _lib.ERR_OOM
    assert f(fake, fake, 1 << 20, 1 << 20, 4, None) == _lib.ERR_OOM
    assert f(None, fake, 8, 8, 4, None) == _lib.ERR_ARG
    assert f(fake, None, 8, 8, 4, None) == _lib.ERR_ARG
    assert f(fake, fake, 0, 8, 4, None) == _lib.ERR_ARG
    assert f(fake, fake, 8, 8, 6, None) == _lib.ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("conn", [4, 8])
def test_noalloc_matches_context_entry_on_consecutive_calls(cuda, conn):
    import torch
    from nscale_gb300 import _lib
    from nscale_gb300.context import get_context, ptr, stream_handle
    L = _lib.load()
    # a large case first, then a smaller one (the array still holds the first
    # call's planes), then one at exactly the maximum size
    cases = [(1536, 2048, 0.62), (333, 517, 0.55), (2048, 2048, 0.6)]
    imgs, wants, gots = [], [], []
    for k, (rows, cols, p) in enumerate(cases):
        img = torch.from_numpy(_mask(rows, cols, 0xF111 + 31 * k + conn, p)).cuda()
        want = torch.empty_like(img)
        ctx = get_context(rows, cols)
        ctx.check(L.nsg_imfill_holes_u8(ctx.h, ptr(img), ptr(want), rows, cols, conn, stream_handle()))
        imgs.append(img)
        wants.append(want)
        gots.append(torch.full_like(img, 7))
    torch.cuda.synchronize()
    # the no-allocation calls back to back on one stream, no host sync between
    for (rows, cols, _), img, got in zip(cases, imgs, gots):
        rc = L.nsg_imfill_holes_u8_noalloc(ptr(img), ptr(got), rows, cols, conn, stream_handle())
        assert rc == 0, L.nsg_status_string(rc)
    torch.cuda.synchronize()
    for k, (img, want, got) in enumerate(zip(imgs, wants, gots)):
        w, g = want.cpu().numpy(), got.cpu().numpy()
        assert (w == 255).sum() > (img.cpu().numpy() == 255).sum()  # some holes were filled
        assert np.array_equal(g, w), f"case {k} {cases[k]}: {(g != w).sum()} pixels differ"
