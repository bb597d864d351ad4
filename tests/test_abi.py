"""The C-ABI library builds, loads without a GPU, exports every symbol that
include/nrc.h declares, and its host-only entry points behave."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "nrc.h")).read()
    return re.findall(r"^NRC_API\s+[\w\s\*]*?\b(nrc_\w+)\s*\(", src, flags=re.M)


def test_exports_every_declared_symbol(nrclib):
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(nrclib, n), n
    from vknrc_gb300 import nrc

    assert sorted(names) == sorted(nrc.EXPORTS)


def test_default_config_is_reference_constants():
    from vknrc_gb300 import nrc

    c = nrc.default_config()
    assert c.train_batch_size == 16384
    assert np.float32(c.learning_rate) == np.float32(0.002)
    assert np.float32(c.beta1) == np.float32(0.9) and np.float32(c.beta2) == np.float32(0.999)
    assert np.float32(c.epsilon) == np.float32(1e-8) and np.float32(c.ema_alpha) == np.float32(0.99)
    assert c.loss_scale == 1.0 and c.use_ema_weights == 0


def test_he_init_host_deterministic_and_distributed():
    from vknrc_gb300 import nrc

    a = nrc.he_init_host(1234)
    b = nrc.he_init_host(1234)
    c = nrc.he_init_host(1235)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert abs(a.mean()) < 0.01 and abs(a.std() - np.sqrt(2 / 64)) < 0.01


def test_status_strings(nrclib):
    assert nrclib.nrc_status_string(0) == b"ok"
    assert b"timed out" in nrclib.nrc_status_string(6)


def test_create_without_device_fails_cleanly():
    import torch

    from vknrc_gb300 import nrc

    if torch.cuda.is_available():
        return
    cfg = nrc.default_config()
    h = ctypes.c_void_p()
    s = nrc.lib().nrc_create(ctypes.byref(cfg), ctypes.byref(h))
    assert s == 3 and not h.value  # NRC_ERROR_NO_DEVICE, no context


def test_null_arguments_rejected(nrclib):
    assert nrclib.nrc_default_config(None) == 1
    assert nrclib.nrc_he_init_host(0, None) == 1
    assert nrclib.nrc_infer(None, None, None, 0, None, 0, None) == 1
    assert nrclib.nrc_destroy(None) == 1
