"""Regenerate vtkm_presets.npz, the colour presets of the volume plot.

The reference accepts every preset name of VTK-m's colour tables
(is_valid_name, ascent_runtime_conduit_to_vtkm_parsing.cpp:176-197). Its
documentation ships a 256-sample rendering of each of them
(src/docs/sphinx/Actions/color_tables/vtkm/<name>.png, 256 x 64 pixels,
every row the same); this script decodes the first row of each image into
256 RGB bytes per preset, keyed by the preset's name. colortable.py turns
them into 256 colour control points at positions i / 255.

Usage: python make_presets.py <root of the Ascent sources>
(or set GVR_REFERENCE_ROOT). The package reads only the committed .npz.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from ascent_gb300.png import decode_png  # noqa: E402

BARS = "src/docs/sphinx/Actions/color_tables/vtkm"


def color_bars(root: Path) -> dict:
    """name -> (256, 3) uint8: the first row of each colour-bar image."""
    out = {}
    for png in sorted((root / BARS).glob("*.png")):
        img = decode_png(png.read_bytes())
        if img.shape[1] != 256 or not (img == img[:1]).all():
            raise ValueError(f"{png.name}: expected 256 identical columns per row")
        out[png.stem] = img[0, :, :3].copy()
    return out


def main(argv) -> None:
    root = argv[1] if len(argv) > 1 else os.environ.get("GVR_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_presets.py <root of the Ascent sources>")
    bars = color_bars(Path(root))
    np.savez_compressed(HERE / "vtkm_presets.npz", **bars)
    print(f"wrote vtkm_presets.npz: {len(bars)} presets")


if __name__ == "__main__":
    main(sys.argv)
