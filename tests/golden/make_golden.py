"""Generate the committed golden fixtures under tests/golden/.

Run in a container that has the reference sources at /root/reference (x86):

    python tests/golden/make_golden.py

* signs_kat.json   - sign bits of the reference's bitHD3Generator
                     (src/Utilities.cpp:21-41) for seeds 42 and 7, drawn with
                     std::default_random_engine (libstdc++), 6144 bits each.
* fwht_ref.npz     - inputs and outputs of the reference's own FFHT
                     fht_float (src/fht.c, compiled from the reference sources
                     by oracle/Makefile target `ref`) for log_n = 1..12.
* search_small.npz - a small end-to-end case (data, queries, parameters) with
                     the oracle's buckets and search results, used to check
                     the GPU library against committed vectors.
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

    # small end-to-end case (config-0 distribution, reduced size)
    n, d, nq = 900, 44, 40
    X = (rng.standard_normal((n, d)) / np.sqrt(d) * rng.lognormal(0, 0.5, (n, 1))).astype(np.float32)
    Q = rng.standard_normal((nq, d)).astype(np.float32)
    D, R, m, s, c, k, seed = 128, 2, 50, 10, 80, 10, 42
    idx = O.CEOs(n, d)
    idx.setIndexParam(D, R, m, 4, seed)
    idx.build_coCEOs_Est(X)
    idx.n_probed_vectors = s
    idx.n_cand = c
    ids, dists = idx.search_coCEOs_Est(Q, k)
    bids, bvals = idx.buckets()
    np.savez_compressed(os.path.join(HERE, "search_small.npz"), X=X, Q=Q,
                        params=np.array([D, R, m, s, c, k, seed], np.int32),
                        bucket_ids=bids, bucket_vals=bvals, ids=ids, dists=dists)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
