"""Regenerate the committed fixtures under tests/golden/ from the reference.

Run where a checkout of the reference is available (GPU machines have none
and use the committed copies), giving the checkout's root directory:

    python tests/golden/make_fixtures.py PATH_TO_REFERENCE_CHECKOUT

It copies the reference's data tables (crates/sky-core/src/data.rs reads
bands.csv, atmosphere_profile.csv, aerosol_profile.csv, aerosol_optics.csv;
spectrum.rs:255 embeds CIE_xyz_1931_2deg.csv) verbatim into tests/golden/data/
and records their SHA-256 in tests/golden/data/SHA256SUMS.  data/mie_phase.csv
is not in the reference checkout (listed in .MISSING_LARGE_BLOBS) and is not
produced here.
"""

from __future__ import annotations

import hashlib
import shutil
import sys
from pathlib import Path

FILES = ("bands.csv", "atmosphere_profile.csv", "aerosol_profile.csv", "aerosol_optics.csv",
         "CIE_xyz_1931_2deg.csv")


def main(reference: str) -> None:
    src = Path(reference) / "data"
    dst = Path(__file__).resolve().parent / "data"
    dst.mkdir(parents=True, exist_ok=True)
    lines = []
    for name in FILES:
        shutil.copyfile(src / name, dst / name)
        digest = hashlib.sha256((dst / name).read_bytes()).hexdigest()
        lines.append(f"{digest}  {name}")
    (dst / "SHA256SUMS").write_text("\n".join(lines) + "\n")
    print(f"wrote {len(FILES)} tables to {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_fixtures.py PATH_TO_REFERENCE_CHECKOUT")
    main(sys.argv[1])
