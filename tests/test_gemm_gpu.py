"""The tcgen05 BF16 GEMM (TMA tiles, TMEM accumulator) against a plain
PyTorch fp32 reference of the same op, for every epilogue and the shapes of
the surrogate's forward and backward passes."""

import ctypes

import pytest
import torch

from optika_gb300 import _lib as L
from optika_gb300._api import ptr, stream_handle

pytestmark = pytest.mark.gpu


def _gemm(a, b, bias, epilogue, k=None, z_in=None, transposed=False):
    m = a.shape[0]
    k = a.shape[1] if k is None else k
    n = b.shape[0]
    lib = L.load()
    err = torch.zeros(1, dtype=torch.int32, device=a.device)
    out_t = None
    if epilogue in (L.EPI_SILU_BF16, L.EPI_DSILU_BF16):
        out = torch.empty((m, n), dtype=torch.bfloat16, device=a.device)
        z = z_in if z_in is not None else torch.empty((m, n), dtype=torch.bfloat16,
                                                      device=a.device)
        if transposed:
            out_t = torch.full((n, m + 8), float("nan"), dtype=torch.bfloat16, device=a.device)
    else:
        out = torch.full((m, n), float("nan"), dtype=torch.float32, device=a.device)
        z = None
    st = lib.otx_gemm_bf16(ptr(a), a.stride(0), ptr(b), b.stride(0), m, n, k,
                           ptr(bias) if bias is not None else None, epilogue, ptr(out), n,
                           ptr(z) if z is not None else None,
                           ptr(out_t) if out_t is not None else None, m + 8, ptr(err),
                           stream_handle())
    assert st == L.OK, lib.otx_status_string(st)
    torch.cuda.synchronize()
    assert err.item() == 0
    if transposed:
        return out, z, out_t
    return out, z


def _pad_k(x, k_pad):
    out = torch.zeros((x.shape[0], k_pad), dtype=x.dtype, device=x.device)
    out[:, : x.shape[1]] = x
    return out


@pytest.mark.parametrize(
    "m,n,k",
    [(300, 256, 256), (128, 3, 256), (1000, 256, 9), (256, 256, 4096), (16, 64, 512),
     (513, 128, 64)],
)
@pytest.mark.parametrize("epilogue", [L.EPI_SILU_BF16, L.EPI_BIAS_F32, L.EPI_F32])
def test_gemm_matches_torch(cuda, m, n, k, epilogue):
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n + k)
    k_store = (k + 7) // 8 * 8  # rows 16-byte aligned
    a = _pad_k(torch.randn((m, k), device="cuda", generator=g).to(torch.bfloat16), k_store)
    b = _pad_k(torch.randn((n, k), device="cuda", generator=g).to(torch.bfloat16), k_store)
    # poison the row padding: the tensor maps cover k columns only, so the
    # kernel must see zeros (TMA fill) there, never these NaNs
    if k_store > k:
        a[:, k:] = float("nan")
        b[:, k:] = float("nan")
    bias = torch.randn(n, device="cuda", generator=g)
    out, z = _gemm(a, b, bias, epilogue, k=k)
    ref = a[:, :k].float() @ b[:, :k].float().T
    tol = 2e-3 * (k ** 0.5)
    if epilogue == L.EPI_F32:
        assert torch.allclose(out, ref, atol=tol, rtol=1e-3)
    elif epilogue == L.EPI_BIAS_F32:
        assert torch.allclose(out, ref + bias, atol=tol, rtol=1e-3)
    else:
        pre = ref + bias
        assert torch.allclose(z.float(), pre, atol=tol + 1e-2 * pre.abs().max().item(), rtol=1e-2)
        act = torch.nn.functional.silu(pre)
        assert torch.allclose(out.float(), act, atol=tol + 1e-2 * act.abs().max().item(), rtol=1e-2)


@pytest.mark.parametrize("m,n,k", [(256, 256, 65536), (3, 256, 70000), (256, 9, 4096),
                                   (200, 64, 128)])
def test_gemm_split_k_atomic(cuda, m, n, k):
    """Weight-gradient shape: small output, K = batch; K split across CTAs
    and summed by float atomics."""
    g = torch.Generator(device="cuda").manual_seed(k + m)
    a = torch.randn((m, k), device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn((n, k), device="cuda", generator=g).to(torch.bfloat16)
    out, _ = _gemm(a, b, None, L.EPI_F32_ATOMIC)
    ref = a.double() @ b.double().T
    assert torch.allclose(out.double(), ref, atol=1e-3 * k ** 0.5, rtol=1e-4)


@pytest.mark.parametrize("m,n,k", [(300, 256, 256), (1000, 256, 3), (129, 64, 64)])
def test_gemm_dsilu_and_transposed_copy(cuda, m, n, k):
    """Backward through SiLU: dZ = (dY W) * silu'(Z), with the transposed
    copy the weight gradient consumes."""
    g = torch.Generator(device="cuda").manual_seed(m + k)
    k_store = (k + 7) // 8 * 8
    a = _pad_k(torch.randn((m, k), device="cuda", generator=g).to(torch.bfloat16), k_store)
    b = _pad_k(torch.randn((n, k), device="cuda", generator=g).to(torch.bfloat16), k_store)
    z = (2 * torch.randn((m, n), device="cuda", generator=g)).to(torch.bfloat16)
    out, _, out_t = _gemm(a, b, None, L.EPI_DSILU_BF16, k=k, z_in=z, transposed=True)
    zf = z.float()
    s = torch.sigmoid(zf)
    ref = (a[:, :k].float() @ b[:, :k].float().T) * s * (1 + zf * (1 - s))
    tol = 2e-3 * (k ** 0.5) + 1e-2 * ref.abs().max().item()
    assert torch.allclose(out.float(), ref, atol=tol, rtol=1e-2)
    assert torch.equal(out_t[:, :m], out.T)
    # forward SiLU with the transposed copy of the activations
    bias = torch.randn(n, device="cuda", generator=g)
    h, zz, h_t = _gemm(a, b, bias, L.EPI_SILU_BF16, k=k, transposed=True)
    assert torch.equal(h_t[:, :m], h.T)


def test_elementwise_training_kernels(cuda):
    lib = L.load()
    g = torch.Generator(device="cuda").manual_seed(1)
    rows, cols = 777, 256
    z = (3 * torch.randn((rows, cols), device="cuda", generator=g)).to(torch.bfloat16)
    dy = torch.randn((rows, cols), device="cuda", generator=g)
    dz = torch.empty_like(z)
    assert lib.otx_silu_backward(ptr(dy), ptr(z), ptr(dz), rows * cols, stream_handle()) == L.OK
    zf = z.float()
    s = torch.sigmoid(zf)
    ref = dy * s * (1 + zf * (1 - s))
    assert torch.allclose(dz.float(), ref, atol=1e-2, rtol=1e-2)

    t = torch.empty((cols, rows + 9), dtype=torch.bfloat16, device="cuda")
    assert lib.otx_transpose_bf16(ptr(z), rows, cols, cols, ptr(t), rows + 9,
                                  stream_handle()) == L.OK
    assert torch.equal(t[:, :rows], z.T)

    cs = torch.empty(cols, device="cuda")
    assert lib.otx_colsum_bf16(ptr(z), rows, cols, cols, ptr(cs), stream_handle()) == L.OK
    assert torch.allclose(cs, zf.sum(0), atol=1e-2, rtol=1e-4)
    # the output layer's case: 3 columns in rows of 8, many rows
    z8 = (3 * torch.randn((70001, 8), device="cuda", generator=g)).to(torch.bfloat16)
    cs3 = torch.empty(3, device="cuda")
    assert lib.otx_colsum_bf16(ptr(z8), 70001, 3, 8, ptr(cs3), stream_handle()) == L.OK
    assert torch.allclose(cs3, z8.float()[:, :3].sum(0), atol=0.1, rtol=1e-4)

    # three Adam steps against the closed form of Kingma and Ba (2015)
    w = torch.randn((rows, cols), device="cuda", generator=g)
    m = torch.zeros_like(w)
    v = torch.zeros_like(w)
    w16 = torch.empty((rows, cols), dtype=torch.bfloat16, device="cuda")
    w16t = torch.empty((cols, rows), dtype=torch.bfloat16, device="cuda")
    wr, mr, vr = w.clone(), m.clone(), v.clone()
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-8
    for step in range(1, 4):
        grad = torch.randn((rows, cols), device="cuda", generator=g)
        assert lib.otx_adam(ptr(w), ptr(m), ptr(v), ptr(grad), rows, cols, lr, b1, b2, eps, step,
                            ptr(w16), cols, ptr(w16t), rows, stream_handle()) == L.OK
        mr = b1 * mr + (1 - b1) * grad
        vr = b2 * vr + (1 - b2) * grad * grad
        wr = wr - lr * (mr / (1 - b1 ** step)) / ((vr / (1 - b2 ** step)).sqrt() + eps)
    torch.cuda.synchronize()
    assert torch.allclose(w, wr, atol=1e-6, rtol=1e-5)
    assert torch.equal(w16, w.to(torch.bfloat16))
    assert torch.equal(w16t, w.to(torch.bfloat16).T)
