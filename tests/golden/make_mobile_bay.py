"""Writes tests/golden/mobile_bay.npz from the reference's only shipped deck, the Mobile Bay case
(GOM_Rv1.1.0/Projects/MB_test/2_baroclinic_test/input/: 18,718 nodes, 35,127 triangles, 5 z-levels,
75 open-boundary cells forced by elevation series, one river cell, salinity and temperature
series).  The deck sets hurricane_flag 1, whose hurricane_ser.inp is missing from the reference,
so the fixture records hurricane_flag 0 (the core takes wind and air pressure from its caller
either way).  Run once where the reference is mounted:

    python tests/golden/make_mobile_bay.py /path/to/reference
"""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from gom_release_gb300.gom_inputs import read_deck  # noqa: E402


def main(reference: str) -> None:
    deck_dir = Path(reference) / "GOM_Rv1.1.0" / "Projects" / "MB_test" / "2_baroclinic_test" / "input"
    data = read_deck(deck_dir, overrides={"hurricane_flag": 0.0})
    data.name = "mobile_bay"
    out = Path(__file__).resolve().parent / "mobile_bay.npz"
    data.to_npz(out)
    print(out, out.stat().st_size, "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
