"""swe_totals_noalloc: the totals entry point for callers that cannot call cudaMalloc
(their device memory belongs to their own allocator, or their loop must not stall on an
allocation).  The caller owns the state and the output buffer - here torch tensors - and
the library uses only its fixed internal scratch array.  Checked through the C ABI
against the allocating swe_totals on the same state and block count, bitwise, twice in a
row (the second call meets the first call's leftovers in the shared scratch); the
device's free memory is the same before and after the calls."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def device_state(torch, h, hu, hv, B, pitch, dtype, eta_form):
    """Copies ghosted host arrays into pitched device tensors (the library's layout)."""
    rows, cols = h.shape
    out = []
    fields = (h + B if eta_form else h, hu, hv, B)
    for a in fields:
        t = torch.zeros((rows, pitch), dtype=dtype, device="cuda")
        t[:, :cols] = torch.from_numpy(np.ascontiguousarray(a)).to(dtype)
        out.append(t)
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_noalloc_totals_match_allocating_entry_point(gpu_lib, sw, problems, precision):
    import torch
    L = sw.lib()
    Nx, Ny = 300, 257
    h, hu, hv, B = problems.random_state(Nx, Ny, seed=17, q_scale=0.2, b_scale=0.05)
    f32 = precision == "fp32_mixed"
    if f32:
        # values exactly representable in FP32 so both paths see the same state
        B = B.astype(np.float32).astype(np.float64)
        eta = (h + B).astype(np.float32).astype(np.float64)
        h = eta - B
        hu = hu.astype(np.float32).astype(np.float64)
        hv = hv.astype(np.float32).astype(np.float64)
    Lx, Ly = 1.0, 1.3
    with sw.Solver(Nx, Ny, Lx, Ly, precision=precision) as s:
        s.upload(h, hu, hv, B)
        want = s.totals()
    dxdy = (Lx / Nx) * (Ly / Ny)
    pitch = (Ny + 4 + 31) // 32 * 32
    dtype = torch.float32 if f32 else torch.float64
    eh, ehu, ehv, eB = device_state(torch, h, hu, hv, B, pitch, dtype, f32)
    out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
    prec = sw._lib.SWE_PRECISION_FP32_MIXED if f32 else sw._lib.SWE_PRECISION_FP64
    # swe_totals's block count: four per SM
    blocks = 4 * torch.cuda.get_device_properties(0).multi_processor_count
    assert blocks <= sw._lib.TOTALS_NOALLOC_MAX_BLOCKS
    want_bits = np.array(want, dtype=np.float64).view(np.uint64)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        st = L.swe_totals_noalloc(eh.data_ptr(), ehu.data_ptr(), ehv.data_ptr(), eB.data_ptr(),
                                  prec, Nx, Ny, pitch, dxdy, blocks, out.data_ptr(), None)
        assert st == sw._lib.SWE_OK
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0  # nothing was allocated
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint64), want_bits), (got, want)
        out.fill_(float("nan"))
        torch.cuda.synchronize()


def test_noalloc_rejects_more_blocks_than_its_scratch(gpu_lib, sw):
    import torch
    L = sw.lib()
    a = torch.zeros((8, 32), dtype=torch.float64, device="cuda")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    too_many = sw._lib.TOTALS_NOALLOC_MAX_BLOCKS + 1
    st = L.swe_totals_noalloc(a.data_ptr(), a.data_ptr(), a.data_ptr(), None,
                              sw._lib.SWE_PRECISION_FP64, 4, 4, 32, 1.0, too_many,
                              out.data_ptr(), None)
    assert st == sw._lib.SWE_ERR_BAD_ARG
