"""A thin torch.autograd.Function over the C ABI's area forward/backward pair
(sbc_area_forward_device / sbc_area_backward_device), as a test binding: a
training loop's view of the library.  Checked with torch.autograd.gradcheck
(central differences of the same forward) and against the host FP64
gradient of the oracle's rings."""
from __future__ import annotations

import numpy as np
import pytest

import area_grad as AG
import sbclip_gen as gen

pytestmark = pytest.mark.gpu


def _binding(torch, clipper):
    class IntersectionArea(torch.autograd.Function):
        """area[p] = signed shoelace area of base_p ∩ overlay_p."""

        @staticmethod
        def forward(ctx, bxy, boff, cxy, coff):
            n = boff.numel() - 1
            area = torch.zeros(n, dtype=torch.float64, device=bxy.device)
            st = torch.zeros(n, dtype=torch.int32, device=bxy.device)
            bxy, cxy = bxy.contiguous(), cxy.contiguous()
            # the library works on its own stream: inputs must be ready
            torch.cuda.synchronize()
            clipper.area_forward_device(n, bxy.data_ptr(), boff.data_ptr(), cxy.data_ptr(),
                                        coff.data_ptr(), area.data_ptr(), st.data_ptr())
            if not bool((st == 0).all()):
                raise RuntimeError("a pair failed")
            ctx.save_for_backward(bxy, boff, cxy, coff)
            return area

        @staticmethod
        def backward(ctx, grad_area):
            bxy, boff, cxy, coff = ctx.saved_tensors
            n = boff.numel() - 1
            g = grad_area.contiguous()
            gb = torch.zeros_like(bxy)
            gc = torch.zeros_like(cxy)
            torch.cuda.synchronize()
            clipper.area_backward_device(n, bxy.data_ptr(), boff.data_ptr(), cxy.data_ptr(),
                                         coff.data_ptr(), g.data_ptr(), gb.data_ptr(),
                                         gc.data_ptr())
            return gb, None, gc, None

    return IntersectionArea.apply


def _tensors(torch, pairs):
    import sbclip
    bxy, boff = sbclip.pack_polygons([b for b, _ in pairs])
    cxy, coff = sbclip.pack_polygons([c for _, c in pairs])
    dev = "cuda:0"
    return (torch.tensor(bxy, device=dev, requires_grad=True), torch.tensor(boff, device=dev),
            torch.tensor(cxy, device=dev, requires_grad=True), torch.tensor(coff, device=dev))


def test_autograd_gradcheck():
    torch = pytest.importorskip("torch")
    import sbclip
    clip = sbclip.Clipper(0)
    try:
        area = _binding(torch, clip)
        pairs = gen.small_pairs(2, seed=4800, lo=5, hi=9)
        bxy, boff, cxy, coff = _tensors(torch, pairs)
        assert torch.autograd.gradcheck(lambda b, c: area(b, boff, c, coff), (bxy, cxy),
                                        eps=1e-7, atol=1e-7, rtol=1e-6)
    finally:
        clip.close()


def test_autograd_matches_host_gradient():
    torch = pytest.importorskip("torch")
    import sbclip
    clip = sbclip.Clipper(0)
    try:
        area = _binding(torch, clip)
        pairs = gen.small_pairs(64, seed=4900)
        bxy, boff, cxy, coff = _tensors(torch, pairs)
        w = torch.linspace(0.5, 2.0, len(pairs), dtype=torch.float64, device="cuda:0")
        a = area(bxy, boff, cxy, coff)
        (a * w).sum().backward()
        gb = bxy.grad.cpu().numpy()
        gc = cxy.grad.cpu().numpy()
        bo, co = boff.cpu().numpy(), coff.cpu().numpy()
        for p, (b, c) in enumerate(pairs):
            want, hb, hc = AG.area_gradient(b, c)
            assert abs(a[p].item() - want) <= 1e-12 * max(1.0, abs(want))
            scale = max(np.abs(hb).max(), np.abs(hc).max(), 1e-300) * w[p].item()
            assert np.abs(gb[bo[p]:bo[p + 1]] - w[p].item() * hb).max() <= 1e-12 * scale
            assert np.abs(gc[co[p]:co[p + 1]] - w[p].item() * hc).max() <= 1e-12 * scale
    finally:
        clip.close()
