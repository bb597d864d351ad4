"""Generates the committed golden vectors in tests/golden/ from the reference's
own CPU code (oracle/_ref/libnrcref.so, built by oracle/ref/build_ref.sh from the
reference tree): NRCRecord.glsl's encoding compiled as C++, and test/main.cpp's
Evaluate(). Run in a machine that has the reference tree:

    bash oracle/build_oracle.sh && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from vknrc_gb300 import synthetic as S  # noqa: E402


def edge_records() -> np.ndarray:
    vals = [0.0, 1e-30, 0.125, 0.25, 0.2500001, 0.5, 0.75, 0.9999999, 1.0]
    rows = []
    for i, v in enumerate(vals):
        r = np.zeros(14, np.float32)
        r[0:3] = [v, 1.0 - v, 0.5 * v]
        r[3:5] = [v, 1.0 - v]
        r[5:7] = [1.0 - v, v]
        r[7] = v
        r[8:14] = v
        rows.append(r)
    # positions outside [0,1], large roughness, negative values
    extra = np.array([
        [-0.3, 3.7, 1000.25, 0.1, 0.9, 0.3, 0.7, 5.0, 2.0, -1.0, 0.0, 0.5, 0.5, 0.5],
        [12345.678, -0.001, 0.333, 1.2, -0.2, 0.0, 1.0, 0.0, 65504.0, 1e-8, 3.0, 0.0, 1.0, 0.25],
    ], np.float32)
    return np.concatenate([np.stack(rows), extra])


def main():
    ref = O.ref_lib()
    if ref is None:
        raise SystemExit("reference library not built (oracle/_ref/libnrcref.so); run oracle/build_oracle.sh")
    rng = S.rng_for(20240223, 0, 0)
    # --- encoding
    rec = np.concatenate([edge_records(), S.inputs(rng, 4096)])
    enc = O.ref_encode(rec)
    dirs = np.concatenate([np.array([[0, 0, 1], [0, 0, -1], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0],
                                     [1e-20, 0, 1], [0.6, 0.8, 0]], np.float32), S.sphere(rng, 504)])
    sph = O.ref_sph_encode(dirs)
    np.savez_compressed(os.path.join(HERE, "encode_golden.npz"), records=rec, encoded=enc, dirs=dirs, sph=sph)
    # --- Evaluate(): the reference test's distributions (test/main.cpp:91-99)
    w_a = rng.uniform(-0.02, 0.02, 20672).astype(np.float16).view(np.uint16)
    x_a = rng.uniform(0.0, 1.0, (1024, 64)).astype(np.float16).view(np.uint16)
    y_a = O.ref_evaluate(w_a, x_a)
    # He-initialised weights (src/VkNRCState.cpp:131-136) on encoded synthetic records
    w_b = rng.normal(0.0, np.sqrt(2.0 / 64.0), 20672).astype(np.float16).view(np.uint16)
    r_b = S.inputs(rng, 1024)
    x_b = O.ref_encode(r_b)
    y_b = O.ref_evaluate(w_b, x_b)
    np.savez_compressed(os.path.join(HERE, "evaluate_golden.npz"), w_uniform=w_a, x_uniform=x_a, y_uniform=y_a,
                        w_he=w_b, records_he=r_b, x_he=x_b, y_he=y_b)
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))


if __name__ == "__main__":
    main()
