"""fest_find_resnorm_noalloc: the handle-free, allocation-free residual norm
on caller-owned device arrays, against fest_find_resnorm on the same block.

Collected last so that it also runs after every other test has used the
library on the same device."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from fest3d import abi
from parity import make_pair, small_case


def _call_noalloc(L, ext, flow, ptrs, out, stream=None):
    return L.fest_find_resnorm_noalloc(C.byref(ext), C.byref(flow), *[C.c_void_p(p) for p in ptrs],
                                       abi.ptr(out), C.c_void_p(stream))


def test_noalloc_rejects_before_device_work():
    """argument and scratch-limit checks come before any CUDA call."""
    L = abi.load()
    buf = np.zeros(8)
    ptrs = [buf.ctypes.data] * 4  # never dereferenced: every call below is rejected first
    out = np.zeros(9)
    flow = abi.make_flow()
    assert _call_noalloc(L, abi.Extent(10, 8, 6, 8), flow, ptrs, out) == abi.FEST_ERR_SCRATCH
    assert _call_noalloc(L, abi.Extent(1, 8, 6, 5), flow, ptrs, out) == abi.FEST_ERR_ARG
    for nv in (1, 4, 6):  # only the Euler/laminar and SST variable sets have scales here
        assert _call_noalloc(L, abi.Extent(10, 8, 6, nv), flow, ptrs, out) == abi.FEST_ERR_ARG
    assert _call_noalloc(L, abi.Extent(10, 8, 6, 5), flow, [0] + ptrs[1:], out) == abi.FEST_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("turb", [False, True])
def test_noalloc_resnorm_matches_handle_resnorm(gpu_lib, turb):
    import torch
    kw = dict(nc=(21, 13, 6), ids=(-3, -4, -5, -4, -10, -10))
    if turb:
        kw.update(turb=True, flow_kw=dict(mu_ref=2e-2, mu_variation="sutherland_law", MInf=0.2))
    ext, flow, scheme, bc, nodes, qp = small_case(**kw)
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    q = h.get_next_solution(blk["qp"].copy(order="F"), 1, 0.5)
    ref = h.resnorm()  # fest_find_resnorm through the handle
    assert O.get_next_solution([blk], 1, 0.5) == 0
    assert np.allclose(ref, O.find_resnorm([blk]), rtol=1e-10, atol=0)

    dev = torch.device("cuda", torch.cuda.current_device())
    arrays = [torch.from_numpy(np.ascontiguousarray(h.get(n).ravel(order="F"))).to(dev)
              for n in ("residue", "F", "G", "H")]
    ptrs = [a.data_ptr() for a in arrays]
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    L = gpu_lib
    for call in range(2):  # the second call reuses the scratch the first left behind
        out = np.zeros(ext.n_var + 1)
        abi.check(_call_noalloc(L, ext, flow, ptrs, out, stream), "fest_find_resnorm_noalloc")
        assert np.allclose(out, ref, rtol=1e-12, atol=1e-300), (call, out, ref)


@pytest.mark.gpu
def test_noalloc_refuses_a_capturing_stream(gpu_lib):
    """a call on a stream under capture returns FEST_ERR_ARG and leaves the
    capture intact: the captured graph (one torch add) replays"""
    import torch
    ext, flow, scheme, bc, nodes, qp = small_case(nc=(9, 7, 6), ids=(-3, -4, -5, -4, -10, -10))
    blk, h = make_pair(ext, flow, scheme, bc, nodes, qp)
    h.get_next_solution(blk["qp"].copy(order="F"), 1, 0.5)
    dev = torch.device("cuda", torch.cuda.current_device())
    arrays = [torch.from_numpy(np.ascontiguousarray(h.get(n).ravel(order="F"))).to(dev)
              for n in ("residue", "F", "G", "H")]
    ptrs = [a.data_ptr() for a in arrays]
    out = np.zeros(ext.n_var + 1)
    # the first call on the device does its setup outside any capture
    abi.check(_call_noalloc(gpu_lib, ext, flow, ptrs, out, torch.cuda.current_stream().cuda_stream), "setup")
    x = torch.zeros(16, device=dev)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            x.add_(1.0)
            rc = _call_noalloc(gpu_lib, ext, flow, ptrs, out, s.cuda_stream)
    assert rc == abi.FEST_ERR_ARG
    g.replay()
    torch.cuda.synchronize()
    assert float(x.sum()) == 16.0  # captured, not run; the replay adds once
