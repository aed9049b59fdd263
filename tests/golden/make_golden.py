"""Regenerate the golden fixtures in this directory from the reference tree.

Usage: python make_golden.py <root of the Ascent sources> (or set
GVR_REFERENCE_ROOT). Tests read only the committed .npz files.

apcomp_volume_partial.npz
    The reference's baseline image of its partial-compositing test
    (src/tests/_baseline_images/apcomp/apcomp_volume_partial.png, produced by
    src/tests/apcomp/t_apcomp_volume_partials.cpp:16-57), decoded to RGBA
    uint8 rows as stored in the PNG (top row first).

vtkm_color_bars.npz
    The reference's 256-sample renderings of VTK-m's colour presets
    (src/docs/sphinx/Actions/color_tables/vtkm/<name>.png, 256 x 64, every
    row the same): the first row of each as (256, 3) uint8, keyed by name.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from ascent_gb300.png import decode_png  # noqa: E402


def main(argv) -> None:
    root = argv[1] if len(argv) > 1 else os.environ.get("GVR_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_golden.py <root of the Ascent sources>")
    ref = Path(root)
    png = ref / "src/tests/_baseline_images/apcomp/apcomp_volume_partial.png"
    img = decode_png(png.read_bytes())
    np.savez_compressed(HERE / "apcomp_volume_partial.npz", rgba=img,
                        source=np.array(str(png.relative_to(ref))))
    print("wrote apcomp_volume_partial.npz", img.shape)
    bars = {}
    for f in sorted((ref / "src/docs/sphinx/Actions/color_tables/vtkm").glob("*.png")):
        im = decode_png(f.read_bytes())
        assert im.shape[1] == 256 and (im == im[:1]).all(), f.name
        bars[f.stem] = im[0, :, :3].copy()
    np.savez_compressed(HERE / "vtkm_color_bars.npz", **bars)
    print(f"wrote vtkm_color_bars.npz: {len(bars)} colour bars")


if __name__ == "__main__":
    main(sys.argv)
