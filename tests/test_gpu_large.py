"""GPU parity at the full sizes of the benchmark configurations, through
libnsg.so against the oracle on the same seeded inputs:

* one 4096 x 4096 H&E tile through segmentNuclei (status, int32 labels,
  bounding boxes, final mask), and two ragged slide-edge tiles (4096 x 1337,
  731 x 4096);
* 4096 x 4096 grey reconstruction, uint8 and float32, 4- and 8-connected
  (Gaussian-smoothed noise mask, marker = mask - 30);
* 4096 x 4096 imfillHoles, bwlabel2 and bwareaopen2 on random discs at 40 %
  foreground with 5 % single-pixel holes;
* the 4096 x 4096 disc-pair chain distanceTransform -> -dist / -FLT_MAX ->
  imhmin -> localMinima -> watershed2, with the domain-parallel flood taken.

These are the sizes where the reconstruction's tile queue, the watershed's
capacity fallbacks and the cluster BFS run at full scale.  Integer, byte and
label outputs are bit-exact; float32 outputs equal as IEEE values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLT_MAX = np.finfo(np.float32).max


def T(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def N(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def he_tile(rows, cols, seed):
    """Config-0 statistics, generated on the device (same generator as the
    benchmark's tiles), returned as a host array."""
    from nscale_gb300 import synth_torch
    return synth_torch.he_tile(rows, cols, seed, device="cuda").cpu().numpy()


def _segment(orc, img):
    import torch
    from nscale_gb300.histological_entities import HistologicalEntities as HE
    st, lab, n, bbox, mask = HE.segmentNuclei(torch.from_numpy(img).cuda(), return_mask=True)
    torch.cuda.synchronize()
    ost, olab, omask, obox, _ = orc.segment_nuclei(img)
    assert st == ost
    np.testing.assert_array_equal(lab.cpu().numpy(), olab)
    np.testing.assert_array_equal(bbox, obox)
    assert n == obox.shape[1]
    if st == 0:
        np.testing.assert_array_equal(mask.cpu().numpy(), omask)
    return st, n


def test_segment_nuclei_4096_tile(cuda, orc):
    st, n = _segment(orc, he_tile(4096, 4096, 0x5EED0000))
    assert st == 0 and n > 1000


@pytest.mark.parametrize("shape,seed", [((4096, 1337), 0x5EED0003), ((731, 4096), 0x5EED0004)])
def test_segment_nuclei_ragged_tiles(cuda, orc, shape, seed):
    st, n = _segment(orc, he_tile(*shape, seed))
    assert st == 0 and n > 100


@pytest.mark.parametrize("conn", [4, 8])
def test_imreconstruct_u8_4096(cuda, orc, conn):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    marker, mask = synth.recon_inputs(4096, 4096, seed=0x5EED0001)
    np.testing.assert_array_equal(N(MO.imreconstruct(T(marker), T(mask), conn)),
                                  orc.imreconstruct(marker, mask, conn))


@pytest.mark.parametrize("conn", [4, 8])
def test_imreconstruct_f32_4096(cuda, orc, conn):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    marker, mask = synth.recon_inputs_f32(4096, 4096, seed=0x5EED0001)
    got = N(MO.imreconstruct(T(marker), T(mask), conn))
    want = orc.imreconstruct(marker, mask, conn)
    assert got.dtype == np.float32
    assert np.array_equal(got, want), f"{int((got != want).sum())} pixels differ"


@pytest.fixture(scope="module")
def disc_mask_4096():
    from nscale_gb300 import synth
    return synth.disc_mask(4096, 4096, seed=0x5EED0001)


@pytest.mark.parametrize("conn", [4, 8])
def test_fill_label_areaopen_4096(cuda, orc, disc_mask_4096, conn):
    from nscale_gb300 import morphologic_operations as MO
    m = disc_mask_4096
    assert 0.3 < (m > 0).mean() < 0.45
    np.testing.assert_array_equal(N(MO.imfillHoles(T(m), True, conn)), orc.imfill_holes(m, conn))
    np.testing.assert_array_equal(N(MO.bwlabel2(T(m), conn)), orc.bwlabel2(m, conn))
    got, cnt = MO.bwareaopen2(T(m), minSize=30, maxSize=5000, connectivity=conn)
    want, wcnt = orc.bwareaopen2(m, 30, 5000, conn)
    np.testing.assert_array_equal(N(got), want)
    assert cnt == wcnt


@pytest.mark.parametrize("conn", [8, 4])
def test_disc_pair_chain_4096(cuda, orc, conn):
    """distanceTransform -> negate/mask -> imhmin -> localMinima ->
    watershed2 on 3000 overlapping disc pairs + 2000 single discs, each stage
    compared with the oracle; the domain-parallel flood must be taken."""
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    m = synth.disc_pairs_mask(4096, 4096, seed=0x5EED0002)
    dist = N(MO.distTransform(T(m)))
    np.testing.assert_array_equal(dist, orc.dist_transform(m))
    distance = np.where(m > 0, -dist, -FLT_MAX).astype(np.float32)
    d2 = N(MO.imhmin(T(distance), 1.0, 8))
    od2 = orc.imhmin(distance, 1.0, 8)
    assert np.array_equal(d2, od2), f"imhmin: {int((d2 != od2).sum())} pixels differ"
    np.testing.assert_array_equal(N(MO.localMinima(T(d2), conn)), orc.local_minima(d2, conn))
    bgr = he_tile(4096, 4096, 0x5EED0000)
    bgr[m == 0] = 0
    got = N(MO.watershed2(T(bgr), T(d2), conn))
    from nscale_gb300.context import get_context, stream_handle
    import ctypes as C
    ctx = get_context(4096, 4096)
    diag = (C.c_int * 16)()
    ctx.check(ctx.L.nsg_watershed_diagnostics(ctx.h, diag, stream_handle()))
    np.testing.assert_array_equal(got, orc.watershed2(bgr, d2, conn))
    assert diag[0] == 0, f"fast path not taken (fallback code {diag[0]})"
