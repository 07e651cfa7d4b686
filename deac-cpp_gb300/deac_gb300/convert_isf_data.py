"""Convert an ISF ``.npz`` (arrays ``tau``, ``isf``, ``error``) into the
binary input of deac.e: the three arrays as float64, one after the other
(the reference's tools/convert_isf_data.py:11-19, and the layout its loader
reads, deac.cpp:2060-2087).

    python -m deac_gb300.convert_isf_data isf.npz isf.bin
"""
from __future__ import annotations

import argparse

import numpy as np


def convert_isf_npz(isf_file_in, isf_file_out) -> np.ndarray:
    """Write ``tau``, ``isf`` and ``error`` of the npz as one float64 block of
    shape (3, n_tau) in C order and return that block.  The three arrays must
    be one-dimensional and of one length."""
    with np.load(isf_file_in) as z:
        arrays = [np.asarray(z[k]) for k in ("tau", "isf", "error")]
    n = arrays[0].shape[0] if arrays[0].ndim == 1 else -1
    if any(a.ndim != 1 or a.shape[0] != n for a in arrays):
        raise ValueError("tau, isf and error must be one-dimensional arrays of one length")
    block = np.zeros((3, n), dtype=np.float64)
    for row, a in enumerate(arrays):
        block[row, :] = a.astype(np.float64)
    with open(isf_file_out, mode="wb") as f:
        block.tofile(f)
    return block


def main(argv=None) -> int:
    parser = argparse.ArgumentParser(description="Convert isf NPZ file to binary file.")
    parser.add_argument("isf_file_in", type=str, help="npz isf file in location")
    parser.add_argument("isf_file_out", type=str, help="binary isf file out location")
    args = parser.parse_args(argv)
    convert_isf_npz(args.isf_file_in, args.isf_file_out)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
