"""Copies two of the reference's own input files into
tests/golden/reference_data/, unchanged, as test vectors for the data-file
readers and the replay tests (they then run where the reference tree is
absent, on the GPU machines too):
  data/mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root
      the Samples tree the reference's driver reads (100 ECAL entries);
  data/EmptyFile.root
      the pulse shape the driver builds its template from.
The third file there, mysample_1000_..., was never closed by its writer and
holds no readable tree; it stays out (the tests that check that the readers
refuse it use the reference tree where it exists).
Each copy's SHA-256 is printed; tests/test_ecal_data_io.py holds them.

Usage: MULTIFIT_REFERENCE_ROOT=<reference tree> python tests/golden/make_reference_data.py
"""
import hashlib
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build_oracle  # noqa: E402

FILES = ["mysample_100_0.000_0.000_10_25.00_10.00_0.00_1.000_1.00_CRRC43_0.00_slew_1.00.root", "EmptyFile.root"]


def main() -> int:
    src = os.path.join(build_oracle.REFERENCE_ROOT, "data")
    out = os.path.join(HERE, "reference_data")
    os.makedirs(out, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(out, f))
        print(f, hashlib.sha256(open(os.path.join(out, f), "rb").read()).hexdigest())
    return 0


if __name__ == "__main__":
    sys.exit(main())
