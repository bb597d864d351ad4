"""The online-training loss curve at the frame's own batch: 1000 frames, each with
four chained training steps of 16,384 freshly drawn records (nrc_train_batches:
one launch per frame, as the reference's frame schedule runs its four train
passes, src/rg/NRCRenderGraph.cpp:57-80), lr 1e-3, beta 0.9 / 0.99, eps 1e-8.
Targets are the fixed smooth field of the inputs times lognormal(0, 1) noise.

The check: an FP64 training pass (tests/fp64_pass.py, float64 torch on the same
GPU: the oracle pass, not the product) runs the same 4,000 steps on the same
records and features from the same initial weights. The GPU's per-record
relative-L2 loss (its FP64 check-path accumulator) is compared with the FP64
pass's: the mean over the last 100 frames within 2% (the stated tolerance for
this path), and the first frame within 1% (identical weights up to their fp16
rounding).

The batched form runs the same check on a cache trained inside one batched
launch (nrc_train_many) beside a second cache with its own records, each with a
43-CTA group (the frame's training split): the served and batched forms train
a cache this way, and its loss stays within the same 2% of the FP64 pass's."""
import numpy as np
import pytest

from gpu_util import count

pytestmark = pytest.mark.gpu

FRAMES = 1000
BATCHES = 4
RECORDS = 16384
LR, BETA1, BETA2, EPS = 1e-3, 0.9, 0.99, 1e-8
TAIL = 100
TOLERANCE = 0.02


@pytest.mark.parametrize("form", ["single", "batched"])
def test_loss_curve_frame_batch_vs_fp64(cuda, form):
    import torch

    import fp64_pass as F
    from vknrc_gb300 import Cache, nrc, synthetic as S

    gen = torch.Generator(device="cuda")
    gen.manual_seed(20241204)
    gpu_loss, ref_loss = [], []
    with Cache(seed=2025, learning_rate=LR, beta1=BETA1, beta2=BETA2, epsilon=EPS, track_loss=1) as c, \
            Cache(seed=2026, learning_rate=LR, beta1=BETA1, beta2=BETA2, epsilon=EPS) as other:
        _, entries = c.get_optimizer()
        ref = F.Fp64Adam(entries[:, 2], LR, BETA1, BETA2, EPS, "cuda")
        counts = [count(RECORDS) for _ in range(BATCHES)]
        other_counts = [count(RECORDS) for _ in range(BATCHES)]
        enc = torch.empty((RECORDS, 64), dtype=torch.int16, device="cuda")
        c.get_loss()  # start from an empty accumulator
        for frame in range(FRAMES):
            recs = [S.train_records_device(gen, RECORDS, target="field", sigma=1.0) for _ in range(BATCHES)]
            for b in range(BATCHES):
                counts[b].fill_(RECORDS)
            if form == "single":
                c.train_batches(recs, counts)
            else:
                other_recs = [S.train_records_device(gen, RECORDS, target="field", sigma=1.0) for _ in range(BATCHES)]
                for b in range(BATCHES):
                    other_counts[b].fill_(RECORDS)
                nrc.train_many([nrc.train_job(c, recs, counts), nrc.train_job(other, other_recs, other_counts)],
                               ctas=[43, 43])
            s, k = c.get_loss()
            assert k == BATCHES * RECORDS
            gpu_loss.append(s / k)
            fl = 0.0
            for r in recs:
                c.encode(r[:, 6:20].contiguous(), counts[0], enc)
                x = enc.view(torch.float16).double()
                fl += float(ref.step(x, r[:, 0:3].double()))
            ref_loss.append(fl / BATCHES)
        assert c.error() == 0 and other.error() == 0

    gpu_loss = np.asarray(gpu_loss)
    ref_loss = np.asarray(ref_loss)
    assert np.all(np.isfinite(gpu_loss))
    # both learn: within a few frames the loss falls to the floor the lognormal
    # noise of the targets sets, far below the first frame's
    assert ref_loss[-TAIL:].mean() < 0.5 * ref_loss[0]
    assert gpu_loss[-TAIL:].mean() < 0.5 * gpu_loss[0]
    first = abs(gpu_loss[0] - ref_loss[0]) / ref_loss[0]
    rel = abs(gpu_loss[-TAIL:].mean() - ref_loss[-TAIL:].mean()) / ref_loss[-TAIL:].mean()
    print(f"\n {form} loss: first frame {gpu_loss[0]:.4g} (fp64 {ref_loss[0]:.4g}, rel {first:.4f}); last-{TAIL} mean "
          f"{gpu_loss[-TAIL:].mean():.4g} (fp64 {ref_loss[-TAIL:].mean():.4g}); rel diff {rel:.4f}")
    assert first <= 0.01
    assert rel <= TOLERANCE
