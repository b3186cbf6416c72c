"""GPU (libnsg.so) against outputs of nscale's OWN code: the fixtures in
tests/golden/nscale_ref_golden.npz were produced by nscale's functions
compiled from its sources (see tests/golden/make_golden.py), so these tests
tie the CUDA path to the reference directly, not only through the oracle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
ALT_PARAMS = dict(T1=2.5, T2=2.0, G1=60, G2=30, minSize=5, maxSize=2000, minSizeSeg=15,
                  fillHolesConnectivity=8, reconConnectivity=4, watershedConnectivity=4)


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(GOLD, "nscale_ref_golden.npz"))


def T(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def N(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("conn", [4, 8])
def test_gpu_recon_and_binary_vs_nscale(cuda, g, conn):
    from nscale_gb300 import morphologic_operations as MO
    np.testing.assert_array_equal(N(MO.imreconstruct(T(g["recon/marker"]), T(g["recon/mask"]), conn)),
                                  g[f"recon/u8_{conn}"])
    assert np.array_equal(N(MO.imreconstruct(T(g["recon/markerf"]), T(g["recon/maskf"]), conn)),
                          g[f"recon/f32_{conn}"])
    bw, seeds = g["bin/bw"], g["bin/seeds"]
    marker = np.where(seeds > 0, bw, 0).astype(np.uint8)
    np.testing.assert_array_equal(N(MO.imfillHoles(T(bw), True, conn)), g[f"bin/fill_{conn}"])
    np.testing.assert_array_equal(N(MO.bwselect(T(bw), T(seeds), conn)), g[f"bin/bwselect_{conn}"])
    np.testing.assert_array_equal(N(MO.imreconstructBinary(T(marker), T(bw), conn)), g[f"bin/reconbin_{conn}"])
    np.testing.assert_array_equal(N(MO.bwlabel2(T(bw), conn)), g[f"bin/bwlabel2_{conn}"])
    o, n = MO.bwareaopen2(T(bw), minSize=30, maxSize=400, connectivity=conn)
    np.testing.assert_array_equal(N(o), g[f"bin/areaopen_{conn}"])
    assert n == int(g[f"bin/areaopen_{conn}_n"])


def test_gpu_distance_chain_vs_nscale(cuda, g):
    from nscale_gb300 import morphologic_operations as MO
    d2 = N(MO.imhmin(T(g["ws/distance"]), 1.0, 8))
    assert np.array_equal(d2, g["ws/distance2"])
    for conn in (4, 8):
        np.testing.assert_array_equal(N(MO.localMinima(T(d2), conn)), g[f"ws/minima_{conn}"])
        np.testing.assert_array_equal(N(MO.watershed2(T(g["ws/bgr"]), T(d2), conn)), g[f"ws/watershed2_{conn}"])


def test_gpu_open_and_pixel_ops_vs_nscale(cuda, g):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300.histological_entities import HistologicalEntities as HE
    img = g["open/img"]
    np.testing.assert_array_equal(N(MO.morphOpen(T(img), MO.disk19().numpy())), g["open/disk19"])
    np.testing.assert_array_equal(N(MO.morphOpen(T(img), MO.cross3().numpy())), g["open/cross3"])
    bgr = g["pixel/bgr"]
    np.testing.assert_array_equal(N(HE.getRBC(T(bgr), 5.0, 4.0)), g["pixel/rbc_5.0"])
    np.testing.assert_array_equal(N(HE.getRBC(T(bgr), 2.5, 2.0)), g["pixel/rbc_2.5"])
    np.testing.assert_array_equal(N(HE.getBackground(T(bgr))[0]), g["pixel/background"])


@pytest.mark.parametrize("key", ["seg_a", "seg_b", "seg_alt", "seg_white", "seg_empty", "seg_likely"])
def test_gpu_segment_nuclei_vs_nscale(cuda, g, key):
    import torch
    from nscale_gb300.histological_entities import HistologicalEntities as HE
    kw = ALT_PARAMS if key == "seg_alt" else {}
    st, lab, n, bbox, mask = HE.segmentNuclei(T(g[f"{key}/img"]), return_mask=True, **kw)
    torch.cuda.synchronize()
    assert st == int(g[f"{key}/status"])
    if st == 0:
        np.testing.assert_array_equal(lab.cpu().numpy(), g[f"{key}/labels"])
        np.testing.assert_array_equal(mask.cpu().numpy(), g[f"{key}/mask"])
