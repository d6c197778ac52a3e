"""Generate the committed golden fixtures under tests/golden/.

Run where the reference sources are (CEOS_REFERENCE, default /root/reference;
x86, because FFHT is x86 inline assembly):

    python tests/golden/make_golden.py

* signs_kat.json   - sign bits of the reference's bitHD3Generator
                     (src/Utilities.cpp:21-41) for seeds 42 and 7, drawn with
                     std::default_random_engine (libstdc++), 6144 bits each.
* fwht_ref.npz     - inputs and outputs of the reference's own FFHT
                     fht_float (src/fht.c, compiled from the reference sources
                     by oracle/Makefile target `ref`) for log_n = 1..12.

The fixtures made by the reference's own index classes are written by
make_reference_golden.py.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def main():
    kat = {}
    for seed in (42, 7):
        bits = O.sign_bits_std(6144, seed)
        kat[str(seed)] = {"n_bits": 6144, "bits": "".join(map(str, bits.tolist())),
                          "ones": int(bits.sum())}
    with open(os.path.join(HERE, "signs_kat.json"), "w") as fh:
        json.dump(kat, fh, indent=1)

    rng = np.random.default_rng(20240315)
    arrays = {}
    for L in range(1, 13):
        rows = 8 if L <= 9 else 2
        x = (rng.standard_normal((rows, 1 << L)) * rng.lognormal(0, 2, (rows, 1))).astype(np.float32)
        y = O.ref_ffht(x)
        if y is None:
            raise SystemExit("reference FFHT could not be built here")
        arrays[f"x{L}"] = x
        arrays[f"y{L}"] = y
    np.savez_compressed(os.path.join(HERE, "fwht_ref.npz"), **arrays)

    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
