"""nrc_train_noalloc: the training step for callers that cannot allocate device
memory (a renderer that sub-allocates every buffer from its own heaps, a process
under a fixed memory budget). It keeps its one piece of scratch, the gradient
partials, in a fixed array inside the library.

Checked through the C ABI against nrc_train on an identically initialised cache,
on two calls in a row. The two paths sum the same per-record gradients in a
different order (64 partials of two tiles each here, 128 of one tile in the
context), so the comparison uses the tolerance of the other training tests."""
import ctypes

import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu


def _noalloc(buffers, recs, cnt, capacity, cfg, d_error=None):
    import torch

    from vknrc_gb300 import nrc

    w, use, ent, st = buffers
    return nrc.lib().nrc_train_noalloc(w, use, ent, st, recs.data_ptr(), cnt.data_ptr(), capacity, ctypes.byref(cfg),
                                       d_error, torch.cuda.current_stream().cuda_stream)


def test_noalloc_matches_context_training(cuda):
    from vknrc_gb300 import Cache, nrc, synthetic as S

    lr = 0.002
    a = Cache(seed=31, deterministic=1)
    b = Cache(seed=31, deterministic=1)
    cfg = nrc.default_config()
    buffers = b.device_buffers()
    assert np.array_equal(a.get_weights(1), b.get_weights(1))
    for call in range(2):
        recs = dev(S.train_records(S.rng_for(40, call), 16384, target="field", sigma=0.5))
        ca, cb = count(20000), count(20000)
        a.train(recs, ca, write_use=True)
        assert _noalloc(buffers, recs, cb, 16384, cfg) == 0
        assert host(ca)[0] == host(cb)[0] == 16384  # count clamped and written back by both
        sa, ea = a.get_optimizer()
        sb, eb = b.get_optimizer()
        assert sa == sb and sa[0] == call + 1
        assert b.error() == 0
        far = np.abs(ea[:, 2] - eb[:, 2]) > 1e-4 * lr
        assert np.mean(far) < 1e-3, np.mean(far)
        assert np.allclose(ea[:, 0], eb[:, 0], rtol=1e-3, atol=1e-6 * np.abs(ea[:, 0]).max())
        wa, wb = a.get_weights(1).view(np.float16).astype(np.float32), b.get_weights(1).view(np.float16).astype(np.float32)
        assert np.mean(wa != wb) < 1e-2
        assert np.array_equal(b.get_weights(0), b.get_weights(1))  # use_weights written
    a.close()
    b.close()


def test_noalloc_rejects_more_records_than_its_scratch(cuda):
    from vknrc_gb300 import Cache, nrc, synthetic as S

    with Cache(seed=32) as c:
        w0 = c.get_weights(1)
        cfg = nrc.default_config(train_batch_size=20000)
        recs = dev(S.train_records(S.rng_for(41), 20000, sigma=0.5))
        assert _noalloc(c.device_buffers(), recs, count(20000), 20000, cfg) == 8  # NRC_ERROR_TOO_LARGE
        assert np.array_equal(c.get_weights(1), w0) and c.get_optimizer()[0][0] == 0
