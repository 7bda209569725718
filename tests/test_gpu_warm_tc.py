"""The warm start's tensor-core row-tile GEMM (tcgen05, TMA-fed operands)
through gops_debug_tc_gemm, against a plain PyTorch FP32 reference of the
same op on the same BF16 inputs.

Both shapes the network uses: layer 2 (out = relu([xa | xb] bt^T + bias),
K = 256, N = 128, with the head w = exp(out . w3 + b3) fused) and the input
gradient (out = xa bt^T, K = 128, N = 256).  Row counts cover a single row,
partial 128-row tiles, and more tiles than SMs (each CTA then walks several
tiles and both of its accumulators).  The kernel accumulates in FP32 in its
own order: an output may differ from the reference by one BF16 unit (2^-7
relative) plus the FP32 accumulation bound K 2^-24 sum|a b| (written as
2^-14 sum|a b| >= 256 x 2^-24 sum|a b|); the head weight exp(u) is checked
against the head of the kernel's own rounded activations with the bound
2^-16 sum|h w3| (>= 128 x 2^-24 sum|h w3|) on u, plus 1e-6 relative."""
import ctypes

import pytest
import torch

from graphops_gb300 import _native

pytestmark = pytest.mark.gpu

ROWS = [1, 127, 128, 129, 1000, 128 * 400 + 37]


def _call(ctx, mode, xa, xb, bt, m, out, bias=None, head=None, w=None):
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    torch.cuda.synchronize()
    rc = ctx._l.gops_debug_tc_gemm(ctx.handle, mode, p(xa), p(xb), p(bt), m, p(out), p(bias), p(head), p(w), p(err))
    assert rc == 0, ctx._l.gops_last_error(ctx.handle)
    assert int(err.item()) == 0, f"handshake timeout code {int(err.item())}"


def _close(got, want, mag):
    g, r = got.float(), want.float()
    bad = (g - r).abs() > (2.0 ** -7) * r.abs() + (2.0 ** -14) * mag
    assert not bool(bad.any()), (int(bad.sum()), float((g - r).abs().max()))


@pytest.mark.parametrize("m", ROWS)
def test_input_grad_shape(m):
    ctx = _native.default_context()
    gen = torch.Generator(device="cuda").manual_seed(m)
    xa = (torch.randn(m, 128, device="cuda", generator=gen) * 0.5).to(torch.bfloat16)
    bt = (torch.randn(256, 128, device="cuda", generator=gen) * 0.1).to(torch.bfloat16)
    out = torch.full((m, 256), float("nan"), dtype=torch.bfloat16, device="cuda")
    _call(ctx, 1, xa, None, bt, m, out)
    ref = xa.float() @ bt.float().t()
    _close(out, ref, xa.float().abs() @ bt.float().abs().t())


@pytest.mark.parametrize("m", ROWS)
def test_layer2_shape_with_head(m):
    ctx = _native.default_context()
    gen = torch.Generator(device="cuda").manual_seed(1000 + m)
    xa = (torch.randn(m, 128, device="cuda", generator=gen) * 0.5).to(torch.bfloat16)
    xb = (torch.randn(m, 128, device="cuda", generator=gen) * 0.5).to(torch.bfloat16)
    bt = (torch.randn(128, 256, device="cuda", generator=gen) * 0.1).to(torch.bfloat16)
    bias = torch.randn(128, device="cuda", generator=gen) * 0.1
    head = torch.randn(129, device="cuda", generator=gen) * 0.2
    out = torch.full((m, 128), float("nan"), dtype=torch.bfloat16, device="cuda")
    w = torch.full((m,), float("nan"), dtype=torch.float32, device="cuda")
    _call(ctx, 0, xa, xb, bt, m, out, bias, head, w)
    x = torch.cat([xa, xb], 1).float()
    ref = torch.relu(x @ bt.float().t() + bias)
    _close(out, ref, x.abs() @ bt.float().abs().t() + bias.abs())
    h = out.double()
    u = (h @ head[:128].double() + float(head[128])).clamp(-20, 20)
    bound = (2.0 ** -16) * (h.abs() @ head[:128].double().abs()) + 1e-6
    rel = (w.double() - torch.exp(u)).abs() / torch.exp(u)
    assert bool((rel <= bound * 1.01 + 1e-6).all()), float(rel.max())


def test_second_call_reuses_the_kernel_state():
    """Two calls in a row with different row counts give the same rows as
    fresh ones (tensor memory freed and reallocated, barriers re-initialised)."""
    ctx = _native.default_context()
    gen = torch.Generator(device="cuda").manual_seed(7)
    xa = (torch.randn(5000, 128, device="cuda", generator=gen) * 0.5).to(torch.bfloat16)
    bt = (torch.randn(256, 128, device="cuda", generator=gen) * 0.1).to(torch.bfloat16)
    a = torch.empty(5000, 256, dtype=torch.bfloat16, device="cuda")
    b = torch.empty(300, 256, dtype=torch.bfloat16, device="cuda")
    _call(ctx, 1, xa, None, bt, 5000, a)
    _call(ctx, 1, xa, None, bt, 300, b)
    assert torch.equal(a[:300], b)
