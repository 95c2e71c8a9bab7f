"""smc_grid_noalloc -- the grid synthesis for callers that cannot allocate.

Some callers own all their device memory through a fixed arena (their
allocator forbids foreign cudaMalloc calls), or run time loops that cannot
afford the device-wide synchronisation cudaMalloc/cudaFree may cause; they
cannot create a model handle, whose buffers are allocated.  This entry point
gives them the Fourier x Chebyshev synthesis with its intermediate array in
one fixed library-wide device array.  The test checks it against the
handle-based smc_transform on two calls in a row (the array is shared, so the
second call must not see leftovers of the first), for the plain and the padded
grid, and that an oversize request is refused.  This file is collected last,
and passes alone in a fresh process as well as after the other tests.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


@pytest.mark.parametrize("Nx,Nz", [(32, 24), (64, 96)])
def test_noalloc_grid_matches_transform_twice(Nx, Nz):
    import torch
    from specmc_gb300 import _lib, api
    from specmc_gb300.config import ConvectionConfig
    _lib.build()
    lib = _lib.load()
    m = api.build_model(ConvectionConfig(viscosity_model="const", Nx=Nx, Nz=Nz))
    Nk = Nx // 2 + 1
    gen = torch.Generator(device="cpu").manual_seed(Nx + Nz)
    stream = torch.cuda.current_stream().cuda_stream
    for padded, kind, Ng in ((0, _lib.SMC_GRID, Nx), (1, _lib.SMC_SYNTH_PAD, 2 * Nx)):
        for call in range(2):
            cf = torch.complex(torch.randn(Nk, Nz, generator=gen, dtype=torch.float64),
                               torch.randn(Nk, Nz, generator=gen, dtype=torch.float64)).cuda()
            ref = torch.empty(Ng, Nz, dtype=torch.float64, device="cuda")
            _lib.check(lib.smc_transform(m._h, kind, ctypes.c_void_p(cf.data_ptr()),
                                         ctypes.c_void_p(ref.data_ptr()), _lib.SMC_DEVICE))
            out = torch.full((Ng, Nz), float("nan"), dtype=torch.float64, device="cuda")
            rc = lib.smc_grid_noalloc(ctypes.c_void_p(cf.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                      Nx, Nz, padded, ctypes.c_void_p(stream))
            assert rc == 0, lib.smc_last_error()
            torch.cuda.synchronize()
            assert torch.isfinite(out).all()
            assert _rel(out, ref) < 1e-13, (padded, call, _rel(out, ref))


def test_noalloc_grid_beyond_the_launch_row_limit():
    """More Fourier modes (Nk = 65,538) and grid rows (Ng = 131,074) than one
    launch dimension holds (65,535): the kernels stride their rows, so the
    whole field is synthesised.  Checked against an FFT synthesis in torch
    (Chebyshev values at the ascending CGL nodes, then irfft * Ng)."""
    import math

    import torch
    from specmc_gb300 import _lib
    _lib.build()
    lib = _lib.load()
    Nx, Nz = 131074, 4
    Nk = Nx // 2 + 1
    gen = torch.Generator(device="cpu").manual_seed(7)
    cf = torch.complex(torch.randn(Nk, Nz, generator=gen, dtype=torch.float64),
                       torch.randn(Nk, Nz, generator=gen, dtype=torch.float64))
    cf /= (1.0 + torch.arange(Nk, dtype=torch.float64))[:, None]
    cf = cf.cuda()
    j = torch.arange(Nz, dtype=torch.float64)
    xi = -torch.cos(math.pi * j / (Nz - 1))                   # 2 z_j - 1
    T = torch.cos(torch.arange(Nz, dtype=torch.float64)[:, None] * torch.arccos(xi)[None, :])
    X = cf @ T.to(torch.complex128).cuda()                     # (Nk, Nz) values per mode
    ref = torch.fft.irfft(X, n=Nx, dim=0) * Nx
    out = torch.full((Nx, Nz), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.smc_grid_noalloc(ctypes.c_void_p(cf.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                              Nx, Nz, 0, ctypes.c_void_p(stream))
    assert rc == 0, lib.smc_last_error()
    torch.cuda.synchronize()
    assert torch.isfinite(out).all()
    assert _rel(out, ref) < 1e-11, _rel(out, ref)


def test_noalloc_rejects_oversize_request():
    import torch
    from specmc_gb300 import _lib
    _lib.build()
    lib = _lib.load()
    Nx, Nz = 2048, 600                         # (Nx/2+1) * Nz = 614,700 > 524,288
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = lib.smc_grid_noalloc(ctypes.c_void_p(dummy.data_ptr()), ctypes.c_void_p(dummy.data_ptr()),
                              Nx, Nz, 0, None)
    assert rc < 0
    assert b"exceeds the fixed scratch" in lib.smc_last_error()
