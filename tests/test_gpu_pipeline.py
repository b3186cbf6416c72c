"""GPU parity tests of the whole segmentNuclei pipeline (through libnsg.so)
against the oracle: statuses, int32 labels (bit-exact) and bounding boxes."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def run_gpu(img, **kw):
    import torch
    from nscale_gb300.histological_entities import HistologicalEntities as HE
    st, lab, n, bbox, mask = HE.segmentNuclei(torch.from_numpy(img).cuda(), return_mask=True, **kw)
    torch.cuda.synchronize()
    return st, lab.cpu().numpy(), n, bbox, mask.cpu().numpy()


def check(orc, img, **kw):
    st, lab, n, bbox, mask = run_gpu(img, **kw)
    p = orc.Params(**kw)
    ost, olab, omask, obox, _ = orc.segment_nuclei(img, p)
    assert st == ost
    np.testing.assert_array_equal(lab, olab)
    np.testing.assert_array_equal(bbox, obox)
    assert n == obox.shape[1]
    if st == 0:
        np.testing.assert_array_equal(mask, omask)
    return st


def test_golden_tiles(cuda, orc):
    g = np.load(os.path.join(GOLD, "seg_small.npz"))
    for key in ("tile_a", "tile_b"):
        st, lab, n, bbox, _ = run_gpu(g[f"{key}/img"])
        assert st == int(g[f"{key}/status"])
        np.testing.assert_array_equal(lab, g[f"{key}/labels"])
        np.testing.assert_array_equal(bbox, g[f"{key}/bbox"])


@pytest.mark.parametrize("shape,seed", [((512, 512), 0x5EED0000), ((300, 517), 0x5EED0003),
                                        ((731, 256), 0x5EED0004), ((64, 64), 0x5EED0005)])
def test_tiles(cuda, orc, shape, seed):
    from nscale_gb300 import synth
    check(orc, synth.he_tile(*shape, seed=seed))


def test_background_statuses(cuda, orc):
    from nscale_gb300 import synth
    assert check(orc, synth.white_tile(128, 96, seed=7)) == 1
    # ~92 % background pixels -> BACKGROUND_LIKELY
    img = synth.white_tile(100, 100, seed=8)
    img[:8, :] = synth.he_tile(8, 100, seed=9)
    assert check(orc, img) in (1, 2)


def test_no_candidates(cuda, orc):
    from nscale_gb300 import synth
    img = synth.he_tile(128, 128, seed=11, n_nuclei=0, n_rbc=0)
    assert check(orc, img) == 3


def test_non_default_parameters(cuda, orc):
    from nscale_gb300 import synth
    img = synth.he_tile(384, 320, seed=0x5EED0006)
    check(orc, img, T1=2.5, T2=2.0, G1=60, G2=30, minSize=5, maxSize=2000, minSizeSeg=15,
          fillHolesConnectivity=8, reconConnectivity=4, watershedConnectivity=4)


def test_repeatable(cuda, orc):
    """Same input, same bytes, 5 times (determinism of the parallel kernels)."""
    from nscale_gb300 import synth
    img = synth.he_tile(256, 256, seed=0x5EED0007)
    first = run_gpu(img)[1]
    for _ in range(4):
        np.testing.assert_array_equal(run_gpu(img)[1], first)
