"""Generates the committed golden vectors in tests/golden/ from the reference's
own code (oracle/_ref/libnrcref.so, built by oracle/ref/build_ref.sh from the
reference tree): NRCRecord.glsl's encoding compiled as C++, test/main.cpp's
Evaluate(), and the training shaders nrc_train_prepare.comp, nrc_optimize.comp
and NN_nv.glsl's relative-L2 loss gradient compiled as C++ (train_golden.npz).
Run in a machine that has the reference tree:

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
    # He-initialised weights (src/VkNRCState.cpp:39-44) on encoded synthetic records
    w_b = rng.normal(0.0, np.sqrt(2.0 / 64.0), 20672).astype(np.float16).view(np.uint16)
    r_b = S.inputs(rng, 1024)
    x_b = O.ref_encode(r_b)
    y_b = O.ref_evaluate(w_b, x_b)
    np.savez_compressed(os.path.join(HERE, "evaluate_golden.npz"), w_uniform=w_a, x_uniform=x_a, y_uniform=y_a,
                        w_he=w_b, records_he=r_b, x_he=x_b, y_he=y_b)
    train_golden(ref)
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))


# The reference's compiled-in hyper-parameters (nrc_optimize.comp:10-11, Constant.glsl:10-15).
REF_HP = dict(learning_rate=0.002, beta1=0.9, beta2=0.999, epsilon=1e-8, ema_alpha=0.99, loss_scale=1.0,
              batch_cap=16384)
PREP_COUNTS = [0, 1, 127, 128, 129, 16383, 16384, 16385, 20000, 0xFFFFFFFF]


def _state_tuple(st):
    return (st.t, st.beta1_t, st.beta2_t, st.alpha_t, st.alpha_t_1)


def train_golden(ref):
    """Golden vectors of the training shaders (the single-step training case: 16,384
    records, lognormal(0, 1.5) targets, He weights)."""
    rng = S.rng_for(20240224, 0, 0)
    # --- prepare: every count from the initial state and from a state 7 steps in
    st_mid = O.OptState(0, 1.0, 1.0, 1.0, 0.0)
    for _ in range(7):
        O.ref_prepare(16384, st_mid)
    prep_in, prep_out, prep_n, prep_groups = [], [], [], []
    for st0 in [(0, 1.0, 1.0, 1.0, 0.0), _state_tuple(st_mid)]:
        for c in PREP_COUNTS:
            st = O.OptState(*st0)
            n, g = O.ref_prepare(c, st)
            prep_in.append(st0)
            prep_out.append(_state_tuple(st))
            prep_n.append(n)
            prep_groups.append(g)
    prep_counts = np.array(PREP_COUNTS * 2, np.uint32)
    # --- the single-step case: He weights, 16,384 records with lognormal(0, 1.5) targets
    n = 16384
    w32 = rng.normal(0.0, np.sqrt(2.0 / 64.0), O.P).astype(np.float32)
    w16 = w32.astype(np.float16).view(np.uint16)
    rec = S.train_records(rng, n, sigma=1.5)
    enc = O.encode(rec[:, 6:])
    pred = O.forward_f32(w16, enc, nthreads=8)  # unclamped outputs, as the gradient pass uses them
    grad = O.train_grad(w16, enc, rec[:, :3], mode=0, nthreads=8)[0].astype(np.float32)
    # --- loss rows: that case's (prediction, target) pairs, then edge pairs
    edge_p = np.array([[0, 0, 0], [-1, -2, -3], [0.5, -0.5, 2.0], [1e-3, 1e-3, 1e-3], [100, 100, 100],
                       [0, 0, 0], [0, 0, 0], [-5, 0.25, 0.0], [3e4, -3e4, 1.0], [0.1, 0.2, 0.3]], np.float32)
    edge_t = np.array([[0, 0, 0], [1, 2, 3], [0.5, 0.5, 0.5], [400.0, 1.0, 0.0], [0, 0, 0],
                       [327.5, 327.52, 327.6], [1e6, 65504.0, 1e-30], [1e3, 0, 5], [0, 0, 0], [0.1, 0.2, 0.3]],
                      np.float32)
    loss_pred = np.concatenate([pred, edge_p])
    loss_target = np.concatenate([rec[:, :3], edge_t])
    loss_rows = O.ref_loss_rows(loss_pred, loss_target, 1.0)
    # --- optimizer: step 1 from the He initialisation on that case's gradient
    st1 = O.OptState(0, 1.0, 1.0, 1.0, 0.0)
    O.ref_prepare(n, st1)
    e_he = np.zeros((O.P, 4), np.float32)
    e_he[:, 2] = w32
    e_he[:, 3] = w32
    e_he_out = e_he.copy()
    w16_he, use16_he = np.zeros(O.P, np.uint16), np.zeros(O.P, np.uint16)
    O.ref_optimize(e_he_out, grad, n, st1, False, w16_he, use16_he)
    # --- optimizer: a state 7 steps in, moments and EMA away from the weights,
    # gradients with NaN / Inf entries, the EMA written to use_weights
    e_mid = np.empty((O.P, 4), np.float32)
    e_mid[:, 0] = rng.normal(0.0, 0.05, O.P)
    e_mid[:, 1] = rng.uniform(0.0, 0.01, O.P)
    e_mid[:, 2] = rng.normal(0.0, 0.2, O.P)
    e_mid[:, 3] = e_mid[:, 2] + rng.normal(0.0, 0.01, O.P).astype(np.float32)
    g_mid = (rng.normal(0.0, 1.0, O.P) * 10.0 ** rng.uniform(-3, 3, O.P)).astype(np.float32)
    g_mid[::997] = np.nan
    g_mid[5::1009] = np.inf
    g_mid[11::1013] = -np.inf
    count_mid = 1000
    st8 = O.OptState(*_state_tuple(st_mid))
    O.ref_prepare(count_mid, st8)
    e_mid_out = e_mid.copy()
    w16_mid, use16_mid = np.zeros(O.P, np.uint16), np.zeros(O.P, np.uint16)
    O.ref_optimize(e_mid_out, g_mid, count_mid, st8, True, w16_mid, use16_mid)
    hp = np.array([REF_HP[k] for k in ("learning_rate", "beta1", "beta2", "epsilon", "ema_alpha", "loss_scale")],
                  np.float32)
    np.savez_compressed(
        os.path.join(HERE, "train_golden.npz"), hparams=hp, batch_cap=np.uint32(REF_HP["batch_cap"]),
        prep_counts=prep_counts, prep_state_in=np.array(prep_in, np.float64),
        prep_state_out=np.array(prep_out, np.float64), prep_n=np.array(prep_n, np.uint32),
        prep_groups=np.array(prep_groups, np.uint32),
        loss_pred=loss_pred, loss_target=loss_target, loss_rows=loss_rows,
        he_w32=w32, he_grad=grad, he_count=np.uint32(n), he_state=np.array(_state_tuple(st1), np.float64),
        he_entries_out=e_he_out, he_w16=w16_he, he_use16=use16_he,
        mid_entries_in=e_mid, mid_grad=g_mid, mid_count=np.uint32(count_mid),
        mid_state_in=np.array(_state_tuple(st_mid), np.float64), mid_state=np.array(_state_tuple(st8), np.float64),
        mid_entries_out=e_mid_out, mid_w16=w16_mid, mid_use16=use16_mid)


if __name__ == "__main__":
    main()
