"""The allocation-free convolution entry point, through the C ABI.

ep_convolve_noalloc serves callers that can't call cudaMalloc: a host that
runs inside a framework owning the device memory pool, or code running
while a CUDA graph is captured.  It must give the same convolution as the
context path: for the density of a solver context, its output with the
coarse-graining kernel wcgk equals the dencg that ep_poten computes
(poten.f90:27-38), within the FP64 field tolerance of the parity tests
(1e-11 relative), on two calls in a row sharing the scratch array.  The
test allocates the device buffers itself (with torch); the entry point
allocates nothing.  This file is collected last on purpose.
"""
import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi
from eff_pot_gb300.build import build

pytestmark = pytest.mark.gpu


def _context_fields(cfg, seed):
    psi = ep.woods_saxon_psi(cfg.nx, cfg.ny, cfg.nz, cfg.xmax, cfg.ymax, cfg.zmax, cfg.n4, seed=seed)
    with ep.Solver(cfg) as s:
        s.start(psi)
        return s.field("den"), s.field("dencg")


def test_noalloc_convolution_matches_poten(oracle):
    torch = pytest.importorskip("torch")
    build()
    _, f = ep.load_library()
    # non-cubic grid with radix 3 and 5 axes, h = 1 A
    cfg = ep.make_config(nx=32, ny=24, nz=40, xmax=16.0, ymax=12.0, zmax=20.0, n4=150.0,
                         core="OTC", icon=_abi.EP_ICON_PERIODIC)
    shape = (cfg.nx, cfg.ny, cfg.nz)
    with oracle.OracleSolver(cfg) as o:
        wcgk = o.form_factors()[1]
    dev = torch.device("cuda", 0)
    d_ker = torch.from_numpy(np.ascontiguousarray(wcgk.ravel(order="F"))).to(dev)
    cases = [_context_fields(cfg, seed) for seed in (3, 4)]
    ins = [torch.from_numpy(np.ascontiguousarray(den.ravel(order="F"))).to(dev) for den, _ in cases]
    outs = [torch.full_like(x, float("nan")) for x in ins]
    stream = torch.cuda.current_stream(dev).cuda_stream
    for d_in, d_out in zip(ins, outs):  # two calls in a row, same scratch
        st = f["convolve_noalloc"](d_in.data_ptr(), d_ker.data_ptr(), d_out.data_ptr(),
                                   cfg.nx, cfg.ny, cfg.nz, stream)
        assert st == _abi.EP_OK
    torch.cuda.synchronize(dev)
    for (den, dencg), d_out in zip(cases, outs):
        got = d_out.cpu().numpy().reshape(shape, order="F")
        err = np.max(np.abs(got - dencg)) / np.max(np.abs(dencg))
        assert err < 1e-11, err
    # grids beyond the fixed scratch are refused with a status code
    st = f["convolve_noalloc"](ins[0].data_ptr(), d_ker.data_ptr(), outs[0].data_ptr(), 128, 128, 128, stream)
    assert st == 8  # EP_ERR_UNSUPPORTED
    st = f["convolve_noalloc"](ins[0].data_ptr(), d_ker.data_ptr(), outs[0].data_ptr(), 33, 24, 40, stream)
    assert st == 2  # EP_ERR_BAD_GRID
