"""The device Float16C encoder (lbm_float16c_encode, the function the step kernels inline; it uses
the hardware's round-toward-zero multiply) against the oracle's restatement of the reference
codec for every 32-bit float pattern, bit for bit.  (Every code's decode: test_gpu_aux.py.)"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from mojo_lbm_gb300 import _capi

pytestmark = pytest.mark.gpu


def test_encode_every_float_pattern():
    chunk = 1 << 26
    lib = _capi.lib()
    x = torch.empty(chunk, dtype=torch.int32, device="cuda")
    out = torch.empty(chunk, dtype=torch.int16, device="cuda")
    base = torch.arange(chunk, dtype=torch.int64, device="cuda")
    bad = 0
    for start in range(0, 1 << 32, chunk):
        x.copy_(((base + start) & 0xFFFFFFFF).to(torch.int64).sub_((base + start >= (1 << 31)).long() << 32))
        _capi.check(lib.lbm_float16c_encode(x.data_ptr(), out.data_ptr(), chunk, None))
        want = oracle.f16c_encode(x.cpu().numpy().view(np.float32))
        bad += int(np.count_nonzero(out.cpu().numpy().view(np.uint16) != want))
    assert bad == 0, f"{bad} float patterns encode differently"
