"""Host transfers (gpe_upload / gpe_download) from pageable and from pinned host
arrays.  Pageable arrays go through the device staging buffer; pinned arrays are
read and written by the pack kernel directly over the host link.  Both give the
same device state and the same host array, bit for bit."""
import ctypes as C

import numpy as np
import pytest
import torch

from spacetime_gb300 import capi, states
from spacetime_gb300.stepper import Stepper

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
@pytest.mark.parametrize("name,comps", [("bcc", 3), ("c15", 1), ("cube", 5)])
def test_pinned_and_pageable_transfers_agree(gpu, name, comps, prec):
    lat = capi.Lattice(name)
    p = capi.make_params(components=comps, precision=prec, dims=(5, 4, 3), block_scale=0.3, dt=1e-4, lattice=lat)
    src = 0.3 * states.random_state(capi.buffer_shape(lat, p), seed=81)
    pinned = torch.from_numpy(src.copy()).pin_memory()
    with Stepper(lat, p) as s:
        s.upload(capi.PSI_EVEN, src)                # pageable: staging copy
        s.upload(capi.PSI_ODD, pinned.numpy())      # pinned: read by the pack kernel
        a = s.download(capi.PSI_EVEN)
        b = s.download(capi.PSI_ODD)
        out = torch.zeros(a.shape, dtype=torch.float64).pin_memory()
        lib, h = s.lib, s._h
        capi.check(lib.gpe_download(h, capi.PSI_ODD, out.numpy().ctypes.data_as(C.POINTER(C.c_double)), out.numel(),
                                    s.stream), "gpe_download")
    assert np.array_equal(a, b)
    assert np.array_equal(out.numpy(), b)
    if prec == capi.FP64:
        interior = (slice(1, -1),) * 3
        assert np.array_equal(b[interior], src[interior])


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32])
def test_transfer_by_dma_agrees(gpu, prec):
    """GPE_TUNE_TRANSFER 1: pinned host arrays go through the staging buffer by DMA
    copies; the device state and the downloaded array equal the direct form's, bit
    for bit, and the setting reads back."""
    lat = capi.Lattice("bcc")
    p = capi.make_params(components=3, precision=prec, dims=(6, 4, 3), block_scale=0.3, dt=1e-4, lattice=lat)
    src = 0.3 * states.random_state(capi.buffer_shape(lat, p), seed=83)
    pinned = torch.from_numpy(src.copy()).pin_memory()
    got = []
    for mode in (0, 1):
        with Stepper(lat, p) as s:
            s.set_tuning(capi.TUNE_TRANSFER, mode)
            assert s.get_tuning(capi.TUNE_TRANSFER) == mode
            s.upload(capi.PSI_ODD, pinned.numpy())
            s.start()
            s.step(3)
            out = torch.zeros(src.shape, dtype=torch.float64).pin_memory()
            s.download(s.current, out=out.numpy())
            got.append(out.numpy().copy())
    assert np.array_equal(got[0], got[1])
    with Stepper(lat, p) as s:
        with pytest.raises(capi.GpeError):
            s.set_tuning(capi.TUNE_TRANSFER, 2)
