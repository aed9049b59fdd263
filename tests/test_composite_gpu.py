"""Device partial compositor (gvr_composite_partials) against the FP32
restatement of PartialCompositor::composite, which is itself pinned byte
for byte to the reference's compiled compositor and its golden image.
Integer/ordering work and an FMA-free FP32 blend: comparisons are exact."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.test_oracle_pins import GOLDEN, _random_partials, apcomp_case, partials_to_png_rgba

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def comp():
    from ascent_gb300 import compositing
    return compositing


def test_golden_image(comp):
    golden = np.load(GOLDEN / "apcomp_volume_partial.npz")["rgba"]
    images, w, h = apcomp_case()
    out = comp.PartialCompositor().composite(images)
    assert np.array_equal(partials_to_png_rgba(out, w, h), golden)
    assert out.tobytes() == O.composite_partials_f32(images).tobytes()


@pytest.mark.parametrize("seed,n_images,ties,density", [(0, 2, False, 0.6), (1, 4, False, 0.6),
                                                        (2, 8, False, 0.9), (3, 3, True, 0.6),
                                                        (4, 1, False, 0.3), (5, 37, False, 0.5)])
def test_random_sets_bit_exact(comp, seed, n_images, ties, density):
    rng = np.random.default_rng(seed)
    ims = _random_partials(rng, n_images, density=density, ties=ties)
    got = comp.PartialCompositor().composite(ims)
    ref = O.composite_partials_f32(ims)
    assert got.tobytes() == ref.tobytes()
    # and within FP32 rounding of the FP64 oracle
    g = got[np.argsort(got["pixel_id"], kind="stable")]
    r64 = O.composite_partials(ims, precision=64)
    np.testing.assert_array_equal(g["pixel_id"], r64["pixel_id"])
    np.testing.assert_allclose(g["rgb"], r64["rgb"], rtol=0, atol=2e-6)


def test_edge_cases(comp):
    pc = comp.PartialCompositor()
    assert len(pc.composite([])) == 0
    assert len(pc.composite([np.zeros(0, comp.PARTIAL_DTYPE)] * 3)) == 0
    one = np.zeros(1, comp.PARTIAL_DTYPE)
    one["pixel_id"], one["alpha"], one["depth"] = 7, 0.25, 3.0
    assert pc.composite([one]).tobytes() == one.tobytes()
    # opaque front record, zero-alpha record, -0/+0 depths, negative ids,
    # one pixel with a long run of records
    rng = np.random.default_rng(11)
    a = np.zeros(2000, comp.PARTIAL_DTYPE)
    a["pixel_id"] = np.where(np.arange(2000) < 1500, 3, rng.integers(-50, 50, 2000))
    a["depth"] = rng.choice(np.array([-0.0, 0.0, 1.0, -2.5], np.float32), 2000)
    a["alpha"] = rng.choice(np.array([0.0, 0.01, 0.3, 1.0], np.float32), 2000)
    a["rgb"] = (rng.uniform(0, 1, (2000, 3)) * a["alpha"][:, None]).astype(np.float32)
    got = pc.composite([a[:700], a[700:]])
    assert got.tobytes() == O.composite_partials_f32([a[:700], a[700:]]).tobytes()


def test_device_resident_large(comp):
    import torch
    rng = np.random.default_rng(7)
    ims = _random_partials(rng, 8, width=512, height=512, density=0.7)
    flat = np.concatenate(ims)
    d = comp.to_device(flat)
    out = comp.from_device(comp.composite_partials_device(d))
    torch.cuda.synchronize()
    assert out.tobytes() == O.composite_partials_f32(ims).tobytes()
    # size-independent properties: one record per covered pixel, unique
    # pixels first, each group in increasing pixel order
    assert len(out) == len(np.unique(flat["pixel_id"]))
    counts = np.bincount(flat["pixel_id"])
    n_unique = int((counts == 1).sum())
    assert np.all(np.diff(out["pixel_id"][:n_unique]) > 0)
    assert np.all(np.diff(out["pixel_id"][n_unique:]) > 0)
    assert np.all(counts[out["pixel_id"][:n_unique]] == 1)


def test_bad_arguments(comp):
    import ctypes as C
    from ascent_gb300 import _native as N
    n_out = C.c_int64(0)
    assert N.lib().gvr_composite_partials(None, 4, None, C.byref(n_out), N.MEM_HOST, None) == \
        N.GVR_ERR_INVALID_ARGUMENT
    assert N.lib().gvr_composite_partials(None, 0, None, C.byref(n_out), 7, None) == \
        N.GVR_ERR_INVALID_ARGUMENT


def test_sparse_pixel_ids_take_the_sorting_path(comp):
    """Ids spread over the whole int range (the dense histogram would be too
    large): same records, same order."""
    rng = np.random.default_rng(13)
    a = np.zeros(6000, comp.PARTIAL_DTYPE)
    ids = rng.integers(-2 ** 31, 2 ** 31 - 1, 1500)
    a["pixel_id"] = rng.choice(ids, 6000)
    a["depth"] = rng.uniform(-5, 5, 6000).astype(np.float32)
    a["alpha"] = rng.uniform(0, 1, 6000).astype(np.float32)
    a["rgb"] = (rng.uniform(0, 1, (6000, 3)) * a["alpha"][:, None]).astype(np.float32)
    ims = [a[:2500], a[2500:]]
    assert comp.PartialCompositor().composite(ims).tobytes() == O.composite_partials_f32(ims).tobytes()


def test_scratch_trim_returns_pooled_memory(comp):
    """The compositor's scratch stays in the library's pool between calls;
    gvr_scratch_trim gives it back, and the next call allocates it again
    with the same result."""
    import torch
    from ascent_gb300 import _native as N
    rng = np.random.default_rng(21)
    ims = _random_partials(rng, 4, density=0.7)
    first = comp.PartialCompositor().composite(ims)
    torch.cuda.synchronize()
    held = N.scratch_trim(0, 1 << 62)   # keep everything: reports the pool size
    assert held > 0
    assert N.scratch_trim(0, 0) == 0
    again = comp.PartialCompositor().composite(ims)
    assert again.tobytes() == first.tobytes()
    assert N.scratch_trim(0, 1 << 62) > 0


@pytest.mark.parametrize("seed,n_images,ties", [(30, 8, False), (31, 3, True), (32, 1, False)])
def test_async_caller_range_bit_exact(comp, seed, n_images, ties):
    """The caller-range path (no host synchronisation, device count) writes
    the same records in the same order as the measured-range path."""
    import torch
    rng = np.random.default_rng(seed)
    ims = _random_partials(rng, n_images, density=0.7, ties=ties)
    flat = np.concatenate(ims)
    lo, hi = int(flat["pixel_id"].min()) - 5, int(flat["pixel_id"].max()) + 7
    d = comp.to_device(flat)
    out, n_out = comp.composite_partials_device_async(d, lo, hi)
    got = comp.from_device(out[: int(n_out.item())])
    assert got.tobytes() == O.composite_partials_f32(ims).tobytes()


def test_async_caller_range_flags_records_outside(comp):
    import torch
    rng = np.random.default_rng(33)
    flat = np.concatenate(_random_partials(rng, 2, density=0.5))
    d = comp.to_device(flat)
    hi = int(flat["pixel_id"].max()) - 1   # the largest id lies outside
    _, n_out = comp.composite_partials_device_async(d, int(flat["pixel_id"].min()), hi)
    assert int(n_out.item()) == -1
    empty = torch.zeros((0, 6), dtype=torch.int32, device="cuda")
    _, n0 = comp.composite_partials_device_async(empty, 0, 10)
    assert int(n0.item()) == 0


def test_dense_path_beyond_one_scan_tile_of_tiles(comp):
    """Pixel ranges above 1024^2 take the three separate scans instead of
    the fused one; both orders and blends equal the restatement."""
    rng = np.random.default_rng(40)
    n = 1_300_000
    p = np.zeros(n, comp.PARTIAL_DTYPE)
    p["pixel_id"] = rng.integers(0, 2_200_000, n)
    p["depth"] = rng.uniform(0, 4, n).astype(np.float32)
    a = rng.uniform(0.01, 1, n).astype(np.float32)
    p["alpha"] = a
    p["rgb"] = (rng.uniform(0, 1, (n, 3)) * a[:, None]).astype(np.float32)
    ims = [p[: n // 2], p[n // 2:]]
    ref = O.composite_partials_f32(ims)
    assert comp.PartialCompositor().composite(ims).tobytes() == ref.tobytes()
    d = comp.to_device(p)
    out, n_out = comp.composite_partials_device_async(d, 0, 2_200_000 - 1)
    assert comp.from_device(out[: int(n_out.item())]).tobytes() == ref.tobytes()
