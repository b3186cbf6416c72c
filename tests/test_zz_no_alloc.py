"""nsg_imfill_holes_u8_noalloc: hole filling for callers that cannot allocate
device memory.  It is checked against nsg_imfill_holes_u8 (the context-based
entry point) and against the oracle's imfillHoles through the C ABI, on
consecutive calls that share the library's static work array, and its
union-find budget is shown to report through its own status word.  This file is collected last so that the test also runs
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
def test_noalloc_matches_context_entry_on_consecutive_calls(cuda, orc, conn):
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
        o = orc.imfill_holes(img.cpu().numpy(), conn)
        assert np.array_equal(g, o), f"case {k} {cases[k]}: {(g != o).sum()} pixels differ from the oracle"


@pytest.mark.gpu
def test_noalloc_timeout_is_reported(cuda, monkeypatch):
    """With a union-find budget of one step (NSG_SPIN_BUDGET, read at each
    call: this entry has no context to carry a budget) every cross-tile union
    on an all-background image runs out; the call returns NSG_ERR_TIMEOUT from
    its own device status word.  The next call, with the default budget, is
    complete and correct (everything reached from the border: all zero)."""
    import torch
    from nscale_gb300 import _lib
    from nscale_gb300.context import ptr, stream_handle
    L = _lib.load()
    img = torch.zeros((256, 256), dtype=torch.uint8, device="cuda")
    out = torch.full_like(img, 7)
    monkeypatch.setenv("NSG_SPIN_BUDGET", "1")
    assert L.nsg_imfill_holes_u8_noalloc(ptr(img), ptr(out), 256, 256, 4, stream_handle()) == _lib.ERR_TIMEOUT
    monkeypatch.delenv("NSG_SPIN_BUDGET")
    assert L.nsg_imfill_holes_u8_noalloc(ptr(img), ptr(out), 256, 256, 4, stream_handle()) == 0
    torch.cuda.synchronize()
    assert int(out.max()) == 0
