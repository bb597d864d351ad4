"""Loss curve over 1000 online training steps, as the reference's renderer
trains: every step draws fresh records (here from the seeded field-target
distribution), runs one fused training step and one Adam update. The GPU's
relative-L2 loss (accumulated in FP64 on the device, check path) is compared
with the FP64 oracle's training loop started from the same weights: FP64
forward/backward (oracle_train_grad_w64) and Adam in FP64 with the reference's
update rule (shader/src/nrc_optimize.comp:32-54) and no fp16 rounding of the
weights. The tolerance is the one stated for this path: the mean loss of the
last 100 steps within 2% of the FP64 oracle's."""
import os

import numpy as np
import pytest

from gpu_util import count, dev

pytestmark = pytest.mark.gpu

STEPS = 1000
RECORDS = 1024
LR, BETA1, BETA2, EPS = 1e-3, 0.9, 0.99, 1e-8
TAIL = 100
TOLERANCE = 0.02


def test_loss_curve_vs_fp64_oracle(cuda, oracle):
    from vknrc_gb300 import Cache, synthetic as S

    threads = os.cpu_count() or 1
    gpu_loss, ref_loss = [], []
    with Cache(seed=2024, learning_rate=LR, beta1=BETA1, beta2=BETA2, epsilon=EPS, track_loss=1) as c:
        _, entries = c.get_optimizer()
        w = entries[:, 2].astype(np.float64)  # the fp32 master weights after He initialisation
        m = np.zeros_like(w)
        v = np.zeros_like(w)
        beta1_t = beta2_t = 1.0
        n = count(RECORDS)
        c.get_loss()  # start from an empty accumulator
        for step in range(STEPS):
            rec = S.train_records(S.rng_for(555, step), RECORDS, target="field", sigma=1.0)
            c.train(dev(rec), n)
            s, k = c.get_loss()
            assert k == RECORDS
            gpu_loss.append(s / k)

            enc = oracle.encode(rec[:, 6:])
            g, loss = oracle.train_grad_w64(w, enc, rec[:, :3], nthreads=threads)
            ref_loss.append(loss / RECORDS)
            g = g / RECORDS
            m = BETA1 * m + (1.0 - BETA1) * g
            v = BETA2 * v + (1.0 - BETA2) * g * g
            beta1_t *= BETA1
            beta2_t *= BETA2
            w = w - LR * (m / (1.0 - beta1_t)) / (np.sqrt(v / (1.0 - beta2_t)) + EPS)
        assert c.error() == 0

    gpu_loss = np.asarray(gpu_loss)
    ref_loss = np.asarray(ref_loss)
    assert np.all(np.isfinite(gpu_loss))
    # both learn: the tail loss is far below the first steps'
    assert ref_loss[-TAIL:].mean() < 0.5 * ref_loss[:10].mean()
    assert gpu_loss[-TAIL:].mean() < 0.5 * gpu_loss[:10].mean()
    # the first step sees identical weights up to their fp16 rounding
    assert abs(gpu_loss[0] - ref_loss[0]) <= 0.01 * ref_loss[0]
    rel = abs(gpu_loss[-TAIL:].mean() - ref_loss[-TAIL:].mean()) / ref_loss[-TAIL:].mean()
    print(f"loss: first {gpu_loss[0]:.4g} (fp64 {ref_loss[0]:.4g}); last-{TAIL} mean "
          f"{gpu_loss[-TAIL:].mean():.4g} (fp64 {ref_loss[-TAIL:].mean():.4g}); rel diff {rel:.4f}")
    assert rel <= TOLERANCE
