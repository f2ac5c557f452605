"""The allocation-free convolution entry point, through the C ABI.

ep_convolve_noalloc serves callers that can't call cudaMalloc: a host that
runs inside a framework owning the device memory pool, or code running
while a CUDA graph is captured.  Its output with the coarse-graining kernel
wcgk must equal the coarse-grained density dencg that the FP64 oracle's
poten computes (poten.f90:27-38) on the same density, within the FP64 field
tolerance of the parity tests (1e-11 relative), on two calls in a row that
share the scratch array.  Grids: a non-cubic one with radix-3 and radix-5
axes, the largest half spectrum the scratch holds (64^3, whose second
half-spectrum buffer ends at the end of the array), and a 320-point axis
(the longest allowed, where the X passes shrink their line count to fit
shared memory).  The test allocates the device buffers itself (with torch);
the entry point allocates nothing.  This file is collected last on purpose.
"""
import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi
from eff_pot_gb300.build import build

pytestmark = pytest.mark.gpu

GRIDS = [  # (nx, ny, nz), (hx, hy, hz) in A, N4
    ((32, 24, 40), (1.0, 1.0, 1.0), 150.0),
    ((64, 64, 64), (0.8, 0.8, 0.8), 500.0),
    ((320, 16, 16), (0.4, 1.6, 1.6), 100.0),
]


def _oracle_fields(oracle, cfg, seed):
    psi = ep.woods_saxon_psi(cfg.nx, cfg.ny, cfg.nz, cfg.xmax, cfg.ymax, cfg.zmax, cfg.n4, seed=seed)
    with oracle.OracleSolver(cfg) as o:
        o.start(psi)
        return o.field("den"), o.field("dencg"), o.form_factors()[1]


@pytest.mark.parametrize("dims,h,n4", GRIDS)
def test_noalloc_convolution_matches_the_oracle(oracle, dims, h, n4):
    torch = pytest.importorskip("torch")
    build()
    _, f = ep.load_library()
    nx, ny, nz = dims
    cfg = ep.make_config(nx=nx, ny=ny, nz=nz, xmax=nx * h[0] / 2, ymax=ny * h[1] / 2, zmax=nz * h[2] / 2,
                         n4=n4, core="OTC", icon=_abi.EP_ICON_PERIODIC)
    cases = [_oracle_fields(oracle, cfg, seed) for seed in (3, 4)]
    wcgk = cases[0][2]
    dev = torch.device("cuda", 0)
    d_ker = torch.from_numpy(np.ascontiguousarray(wcgk.ravel(order="F"))).to(dev)
    ins = [torch.from_numpy(np.ascontiguousarray(den.ravel(order="F"))).to(dev) for den, _, _ in cases]
    outs = [torch.full_like(x, float("nan")) for x in ins]
    stream = torch.cuda.current_stream(dev).cuda_stream
    for d_in, d_out in zip(ins, outs):  # two calls in a row, same scratch
        st = f["convolve_noalloc"](d_in.data_ptr(), d_ker.data_ptr(), d_out.data_ptr(), nx, ny, nz, stream)
        assert st == _abi.EP_OK
    torch.cuda.synchronize(dev)
    for (den, dencg, _), d_out in zip(cases, outs):
        got = d_out.cpu().numpy().reshape(dims, order="F")
        err = np.max(np.abs(got - dencg)) / np.max(np.abs(dencg))
        assert err < 1e-11, err


def test_noalloc_refuses_what_the_scratch_cannot_hold():
    """Grids past the fixed scratch come back as EP_ERR_UNSUPPORTED, bad
    grids as EP_ERR_BAD_GRID, before any device work."""
    torch = pytest.importorskip("torch")
    build()
    _, f = ep.load_library()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    stream = torch.cuda.current_stream(dev).cuda_stream
    assert f["convolve_noalloc"](p, p, p, 128, 128, 128, stream) == _abi.EP_ERR_UNSUPPORTED
    assert f["convolve_noalloc"](p, p, p, 32, 384, 8, stream) == _abi.EP_ERR_UNSUPPORTED
    assert f["convolve_noalloc"](p, p, p, 33, 24, 40, stream) == _abi.EP_ERR_BAD_GRID
    assert f["convolve_noalloc"](p, p, p, 32, 28, 40, stream) == _abi.EP_ERR_BAD_GRID
    torch.cuda.synchronize(dev)
    assert torch.all(buf == 0)
