"""Denoiser kernels against float64 references of the same ops on the same
BF16-valued tensors (every BF16 input is exact in float64, so the reference
carries no rounding of its own), plus a short training run on path-traced
data.

Tolerances, per element, with S = the sum of |a*b| over the K products that
make up that output element (the scale FP32 accumulation error grows with):
  * FP32 outputs (logits, data gradient, weight and bias gradients):
    |out - ref| <= 1e-4 * S;
  * BF16 outputs (ReLU activations, logit gradients): the same plus the BF16
    rounding of the result, 2^-8 * |ref|.
A wrong tap, a dropped 16-channel K slice or a misplaced pixel moves an
element by a few percent of S and fails these bounds.
"""

import ctypes

import numpy as np
import pytest

from vk_cinematic_gb300 import gbsp, scenes

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4
BF16_REL = 2.0 ** -8


def _wt(w):
    """(9, Cout, Cin) -> conv2d weight (Cout, Cin, 3, 3), float64."""
    _, cout, cin = w.shape
    return w.double().reshape(3, 3, cout, cin).permute(2, 3, 0, 1).contiguous()


def ref_conv(x, w, b=None):
    """x (B,H,W,Cin), w (9,Cout,Cin) -> (y, S) as (B,H,W,Cout) float64: y the
    exact convolution (zero padding) plus bias, S the sum of |x*w| (+ |bias|)."""
    import torch

    F = torch.nn.functional
    xd = x.double().permute(0, 3, 1, 2)
    wd = _wt(w)
    bd = None if b is None else b.double()
    y = F.conv2d(xd, wd, bd, padding=1)
    sa = F.conv2d(xd.abs(), wd.abs(), None if bd is None else bd.abs(), padding=1)
    return y.permute(0, 2, 3, 1), sa.permute(0, 2, 3, 1)


def ref_grads(x, w, d):
    """Gradients of sum(conv(x, w, b) * d) in float64: (dW (9,Cout,Cin), dB,
    dX (B,H,W,Cin)) with their sums of |products| (same shapes)."""
    import torch

    G = torch.nn.grad
    xd = x.double().permute(0, 3, 1, 2)
    dd = d.double().permute(0, 3, 1, 2)
    wd = _wt(w)

    def back(t):  # (Cout, Cin, 3, 3) -> (9, Cout, Cin)
        cout, cin = t.shape[0], t.shape[1]
        return t.permute(2, 3, 0, 1).reshape(9, cout, cin)

    dw = back(G.conv2d_weight(xd, wd.shape, dd, padding=1))
    dw_s = back(G.conv2d_weight(xd.abs(), wd.shape, dd.abs(), padding=1))
    db = dd.sum(dim=(0, 2, 3))
    db_s = dd.abs().sum(dim=(0, 2, 3))
    dx = G.conv2d_input(xd.shape, wd, dd, padding=1).permute(0, 2, 3, 1)
    dx_s = G.conv2d_input(xd.shape, wd.abs(), dd.abs(), padding=1).permute(0, 2, 3, 1)
    return (dw, dw_s), (db, db_s), (dx, dx_s)


def within(out, ref, scale, bf16=False, tol=FP32_TOL, bf16_rel=BF16_REL):
    """(worst ratio of |out - ref| to its allowed bound, ok) per element."""
    out = out.double()
    bound = tol * scale + (bf16_rel * ref.abs() if bf16 else 0.0) + 1e-30
    r = ((out - ref).abs() / bound).max().item()
    return r, r <= 1.0


@pytest.mark.parametrize("cin,cout,epi", [(16, 48, 0), (48, 48, 0), (48, 32, 1), (48, 48, 2),
                                          (32, 48, 2)])
def test_conv3x3_forward_matches_torch(gpu_lib, cin, cout, epi):
    import torch

    from vk_cinematic_gb300.denoiser import _ptr, _stream, from_planar, to_planar

    torch.manual_seed(cin * 100 + cout + epi)
    B, H, W = 2, 9, 70
    x = torch.randn((B, H, W, cin), device="cuda").to(torch.bfloat16)
    xp = to_planar(x)
    w = (torch.randn((9, cout, cin), device="cuda") * 0.2).to(torch.bfloat16)
    bias = torch.randn(cout, device="cuda")
    L = gbsp.load()
    if epi == 0:
        out = torch.empty((B, H, cout // 8, W, 8), dtype=torch.bfloat16, device="cuda")
        rc = L.gbsp_dn_conv3x3_forward(_stream(), _ptr(xp), B, H, W, cin, _ptr(w), _ptr(bias),
                                       cout, epi, _ptr(out), None)
    elif epi == 1:
        out = torch.empty((B, H, W, cout), dtype=torch.float32, device="cuda")
        rc = L.gbsp_dn_conv3x3_forward(_stream(), _ptr(xp), B, H, W, cin, _ptr(w), _ptr(bias),
                                       cout, epi, None, _ptr(out))
    else:
        out = torch.empty((B, H, cout // 8, W, 8), dtype=torch.float32, device="cuda")
        rc = L.gbsp_dn_conv3x3_forward(_stream(), _ptr(xp), B, H, W, cin, _ptr(w), None, cout,
                                       epi, None, _ptr(out))
    assert rc == 0, L.gbsp_last_error_string()
    torch.cuda.synchronize()
    ref, S = ref_conv(x, w, bias if epi != 2 else None)
    if epi == 0:
        ref = torch.relu(ref)
    r, ok = within(out if epi == 1 else from_planar(out), ref, S, bf16=epi == 0)
    print(f"mma.sync conv {cin}->{cout} epi {epi}: worst error / bound {r:.3f}")
    assert ok


@pytest.mark.parametrize("cin,cout,epi", [(16, 48, 0), (48, 48, 0), (48, 32, 1), (48, 48, 2),
                                          (32, 48, 2)])
@pytest.mark.parametrize("B,H,W", [(2, 5, 128), (2, 5, 200), (1, 300, 1000)])
def test_conv3x3_tcgen05_matches_torch_and_mma(gpu_lib, cin, cout, epi, B, H, W):
    """The tcgen05 convolution (accumulator in tensor memory) against torch and
    against the mma.sync kernel; W = 200 leaves a partial 128-pixel tile, the
    300-row image gives every CTA strips of 8 rows (the row ring wraps)."""
    import torch

    from vk_cinematic_gb300.denoiser import _ptr, _stream, from_planar, to_planar

    torch.manual_seed(cin * 100 + cout + epi + W)
    x = torch.randn((B, H, W, cin), device="cuda").to(torch.bfloat16)
    xp = to_planar(x)
    w = (torch.randn((9, cout, cin), device="cuda") * 0.2).to(torch.bfloat16)
    bias = torch.randn(cout, device="cuda")
    L = gbsp.load()
    outs = []
    for fn in (L.gbsp_dn_conv3x3_forward_tc, L.gbsp_dn_conv3x3_forward):
        if epi == 0:
            out = torch.full((B, H, cout // 8, W, 8), 7.0, dtype=torch.bfloat16, device="cuda")
            rc = fn(_stream(), _ptr(xp), B, H, W, cin, _ptr(w), _ptr(bias), cout, epi, _ptr(out),
                    None)
            out = from_planar(out)
        elif epi == 1:
            out = torch.full((B, H, W, cout), 7.0, dtype=torch.float32, device="cuda")
            rc = fn(_stream(), _ptr(xp), B, H, W, cin, _ptr(w), _ptr(bias), cout, epi, None,
                    _ptr(out))
        else:
            out = torch.full((B, H, cout // 8, W, 8), 7.0, dtype=torch.float32, device="cuda")
            rc = fn(_stream(), _ptr(xp), B, H, W, cin, _ptr(w), None, cout, epi, None, _ptr(out))
            out = from_planar(out)
        assert rc == 0, L.gbsp_last_error_string()
        outs.append(out)
    torch.cuda.synchronize()
    st = ctypes.c_uint32(0)
    assert L.gbsp_dn_status(ctypes.byref(st)) == 0, st.value
    ref, S = ref_conv(x, w, bias if epi != 2 else None)
    if epi == 0:
        ref = torch.relu(ref)
    r, ok = within(outs[0], ref, S, bf16=epi == 0)
    # the two kernels: each within its bound of the exact result, hence of each
    # other (two BF16 roundings of nearly equal values differ by one BF16 ulp)
    r2, ok2 = within(outs[0], outs[1].double(), 2 * S, bf16=epi == 0, bf16_rel=2 * BF16_REL)
    print(f"tcgen05 conv {cin}->{cout} epi {epi} {B}x{H}x{W}: worst error / bound {r:.3f}, "
          f"vs mma.sync {r2:.3f}")
    assert ok and ok2


@pytest.mark.parametrize("wgrad,shape", [("mma", (2, 12, 67)), ("simt", (2, 12, 67)),
                                         ("mma", (1, 37, 250)), ("mma", (3, 1, 1)),
                                         ("tcgen05", (2, 12, 67)), ("tcgen05", (1, 37, 250)),
                                         ("tcgen05", (3, 1, 1)), ("tcgen05", (4, 40, 200))])
def test_conv_gradients_match_autograd(gpu_lib, wgrad, shape):
    import torch

    from vk_cinematic_gb300.denoiser import KPCNN, from_planar, to_planar

    torch.manual_seed(3)
    net = KPCNN(seed=1, wgrad=wgrad)
    B, H, W = shape
    for li in (0, 1, 7):
        cin, cout, _ = [(16, 48, 0), (48, 48, 0)] [min(li, 1)] if li < 7 else (48, 32, 1)
        x = torch.randn((B, H, W, cin), device="cuda").to(torch.bfloat16)
        d = (torch.randn((B, H, W, cout), device="cuda") * 0.1).to(torch.bfloat16)
        dw = torch.zeros((9, cout, cin), device="cuda")
        db = torch.zeros(cout, device="cuda")
        net.weight_grad(li, to_planar(x), to_planar(d), dw, db)
        torch.cuda.synchronize()
        (rw, sw), (rb, sb), (rx, sx) = ref_grads(x, net.wb[li], d)
        r_w, ok_w = within(dw, rw, sw)
        r_b, ok_b = within(db, rb, sb)
        print(f"{wgrad} {shape} layer {li}: worst error / bound dW {r_w:.3f}, dB {r_b:.3f}")
        assert ok_w and ok_b
        if li > 0:
            dx = from_planar(net.data_grad(li, to_planar(d)))
            torch.cuda.synchronize()
            r_x, ok_x = within(dx, rx, sx)
            print(f"layer {li}: worst error / bound dX {r_x:.3f}")
            assert ok_x


def test_filter_and_relmse_gradient_match_autograd(gpu_lib):
    import torch

    from vk_cinematic_gb300.denoiser import KPCNN, _ptr, _stream, from_planar

    torch.manual_seed(5)
    B, H, W = 2, 7, 9
    logits = torch.randn((B, H, W, 32), device="cuda")
    noisy = torch.rand((B, H, W, 4), device="cuda") * 3
    target = torch.rand((B, H, W, 4), device="cuda") * 2
    net = KPCNN(seed=0)
    out = net.filter(logits, noisy)
    dlog = torch.empty((B, H, 4, W, 8), dtype=torch.bfloat16, device="cuda")
    loss = torch.zeros(1, device="cuda")
    L = gbsp.load()
    assert L.gbsp_dn_relmse_backward(_stream(), _ptr(logits), _ptr(noisy), _ptr(target), B, H, W,
                                     _ptr(dlog), _ptr(loss)) == 0
    dlog = from_planar(dlog)
    # float64 reference
    lr = logits[..., :25].double().clone().requires_grad_(True)
    wts = torch.softmax(lr, dim=-1)
    pad = torch.nn.functional.pad(noisy[..., :3].double().permute(0, 3, 1, 2), (2, 2, 2, 2),
                                  mode="replicate")
    acc = torch.zeros((B, 3, H, W), dtype=torch.float64, device="cuda")
    for k in range(25):
        ky, kx = k // 5, k % 5
        acc = acc + wts[..., k].unsqueeze(1) * pad[:, :, ky:ky + H, kx:kx + W]
    ref_out = acc.permute(0, 2, 3, 1)
    t3 = target[..., :3].double()
    ref_loss = ((ref_out - t3) ** 2 / (t3 * t3 + 0.01)).mean()
    ref_loss.backward()
    torch.cuda.synchronize()
    # filter: a 25-term weighted sum of positive radiance, S = ref_out itself
    r_o, ok_o = within(out[..., :3], ref_out.detach(), ref_out.detach().abs())
    assert ok_o, r_o
    assert abs(loss.item() / (3 * B * H * W) - ref_loss.item()) <= 1e-4 * ref_loss.item()
    # dLogits: w_k (g_k - sum_j w_j g_j) with g the per-tap loss gradient; scale
    # it by w_k (|g_k| + sum_j w_j |g_j|), here bounded by the largest gradient
    g = lr.grad
    r_g, ok_g = within(dlog[..., :25], g, g.abs().amax(dim=-1, keepdim=True).expand_as(g),
                       bf16=True)
    print(f"filter worst error / bound {r_o:.3f}, dLogits {r_g:.3f}")
    assert ok_g
    assert torch.all(dlog[..., 25:] == 0)


def test_adam_matches_torch(gpu_lib):
    import torch

    from vk_cinematic_gb300.denoiser import _ptr, _stream

    torch.manual_seed(0)
    p = torch.randn(1000, device="cuda")
    p_ref = p.clone().requires_grad_(True)
    opt = torch.optim.Adam([p_ref], lr=1e-3)
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    pb = torch.empty(1000, dtype=torch.bfloat16, device="cuda")
    L = gbsp.load()
    for step in range(1, 4):
        g = torch.randn(1000, device="cuda")
        p_ref.grad = g.clone()
        opt.step()
        assert L.gbsp_dn_adam(_stream(), _ptr(p), _ptr(pb), _ptr(g), _ptr(m), _ptr(v),
                              ctypes.c_uint64(1000), ctypes.c_float(1e-3), ctypes.c_float(0.9),
                              ctypes.c_float(0.999), ctypes.c_float(1e-8),
                              ctypes.c_uint32(step)) == 0
    torch.cuda.synchronize()
    assert torch.allclose(p, p_ref.detach(), rtol=1e-5, atol=1e-6)
    assert torch.allclose(pb.float(), p, rtol=1e-2, atol=1e-2)


def test_short_training_reduces_loss(gpu_lib):
    import torch

    from vk_cinematic_gb300 import denoiser

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    rt = gbsp.Runtime(0, stream=stream.cuda_stream)
    noisy, aov, target = denoiser.make_dataset(rt, n_scenes=2, crops_per_scene=2, crop=64,
                                               spp_in=4, spp_ref=256, n_spheres=64, level=3)
    net = denoiser.KPCNN(seed=0)
    feats = net.features(noisy, aov)
    losses = [float(net.train_step(feats, noisy, target, lr=1e-3).item()) for _ in range(60)]
    print("loss", losses[0], "->", losses[-1])
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.8 * losses[0]
    den = net.denoise(noisy, aov)
    assert torch.isfinite(den).all()
    torch.cuda.set_stream(torch.cuda.default_stream())


def test_tile_fallback_serves_bad_tiles_from_plain_samples(gpu_lib):
    """gbsp_dn_tile_fallback: a tile where the 'denoised' image is wrong is
    detected from two independent plain renders and replaced by their mean;
    tiles where it is right keep it."""
    import torch

    from vk_cinematic_gb300.denoiser import _ptr, _stream

    g = torch.Generator(device="cuda").manual_seed(5)
    B, H, W, tile = 2, 40, 56, 16
    mu = torch.full((B, H, W, 4), 1.0, device="cuda")
    A = mu + 0.3 * torch.randn((B, H, W, 4), device="cuda", generator=g)
    C = mu + 0.3 * torch.randn((B, H, W, 4), device="cuda", generator=g)
    D = mu.clone()
    D[1, 16:32, 32:48, :3] += 2.0  # one wrong tile: image 1, tile row 1, column 2
    out = torch.empty_like(D)
    tiles = B * ((H + tile - 1) // tile) * ((W + tile - 1) // tile)
    err = torch.empty(tiles, dtype=torch.float32, device="cuda")
    flags = torch.empty(tiles, dtype=torch.int32, device="cuda")
    L = gbsp.load()
    rc = L.gbsp_dn_tile_fallback(_stream(), _ptr(D), _ptr(A), _ptr(C), B, H, W, tile,
                                 ctypes.c_float(0.05), _ptr(out), _ptr(err), _ptr(flags))
    assert rc == 0, L.gbsp_last_error_string()
    torch.cuda.synchronize()
    f = flags.cpu().numpy().reshape(B, 3, 4)
    bad = np.zeros((B, 3, 4), bool)
    bad[1, 1, 2] = True
    print("tile estimates", err.cpu().numpy().round(3).reshape(B, 3, 4))
    assert np.array_equal(f.astype(bool), bad)
    o = out.cpu()
    assert torch.equal(o[1, 16:32, 32:48, :3], (0.5 * (A + C))[1, 16:32, 32:48, :3].cpu())
    keep = torch.ones((B, H, W), dtype=torch.bool)
    keep[1, 16:32, 32:48] = False
    assert torch.equal(o[..., :3][keep], D.cpu()[..., :3][keep])


@pytest.mark.parametrize("wgrad", ["mma", "tcgen05"])
def test_tensor_core_weight_grad_is_deterministic(gpu_lib, wgrad):
    """The tensor-core weight gradients add their per-CTA partial sums in a fixed
    order: two calls on the same inputs give bit-identical dW and dBias."""
    import torch

    from vk_cinematic_gb300.denoiser import KPCNN, to_planar

    torch.manual_seed(5)
    net = KPCNN(seed=2, wgrad=wgrad)
    B, H, W, cin, cout = 2, 64, 96, 48, 48
    x = to_planar(torch.randn((B, H, W, cin), device="cuda").to(torch.bfloat16))
    d = to_planar((torch.randn((B, H, W, cout), device="cuda") * 0.1).to(torch.bfloat16))
    outs = []
    for _ in range(2):
        dw = torch.zeros((9, cout, cin), device="cuda")
        db = torch.zeros(cout, device="cuda")
        net.weight_grad(1, x, d, dw, db)
        outs.append((dw, db))
    torch.cuda.synchronize()
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("B,H,W", [(1, 37, 200), (2, 4, 129), (1, 1, 3)])
def test_fused_logits_and_filter_match_unfused(gpu_lib, B, H, W):
    """The logits conv fused with the kernel-prediction filter gives the same
    bits as the logits conv followed by the separate filter kernel."""
    import torch

    from vk_cinematic_gb300.denoiser import KPCNN

    torch.manual_seed(11 + W)
    net = KPCNN(seed=4)
    rad = torch.rand((B, H, W, 4), device="cuda") * 3.0
    aov = torch.rand((B, H, W, 8), device="cuda")
    fused = net.denoise(rad, aov)
    logits, _ = net.forward(net.features(rad, aov))
    unfused = net.filter(logits, rad)
    torch.cuda.synchronize()
    assert torch.equal(fused, unfused)


def test_tile_fallback_ignores_noise_alone(gpu_lib):
    """A correct denoised tile checked against very noisy plain renders: the point
    estimates scatter around 0 and often exceed the bound, but a tile falls
    back only when the bound lies two standard errors below its estimate."""
    import torch

    from vk_cinematic_gb300.denoiser import _ptr, _stream

    g = torch.Generator(device="cuda").manual_seed(9)
    B, H, W, tile, bound = 4, 64, 64, 16, 0.01
    mu = torch.full((B, H, W, 4), 1.0, device="cuda")
    A = mu + torch.randn((B, H, W, 4), device="cuda", generator=g)
    C = mu + torch.randn((B, H, W, 4), device="cuda", generator=g)
    D = mu.clone()
    out = torch.empty_like(D)
    tiles = B * (H // tile) * (W // tile)
    err = torch.empty(tiles, dtype=torch.float32, device="cuda")
    flags = torch.empty(tiles, dtype=torch.int32, device="cuda")
    L = gbsp.load()
    rc = L.gbsp_dn_tile_fallback(_stream(), _ptr(D), _ptr(A), _ptr(C), B, H, W, tile,
                                 ctypes.c_float(bound), _ptr(out), _ptr(err), _ptr(flags))
    assert rc == 0, L.gbsp_last_error_string()
    torch.cuda.synchronize()
    above = float((err > bound).float().mean())
    fell = float(flags.float().mean())
    print(f"tiles with estimate above the bound {above:.2f}, fell back {fell:.2f}")
    assert above >= 0.25 and fell <= 0.1


def test_tile_check_flags_bad_tiles_and_sizes_the_fallback(gpu_lib):
    """gbsp_dn_tile_check on synthetic frames with known noise: a tile where D
    is wrong is flagged, correct tiles are not, and the plain spp it asks for
    follows the per-sample variance (sigma^2 = 0.36 per value at mean 1, so
    relMSE 0.01 needs 0.36 / 1.01 / 0.01 = 36 samples, times the margin; the
    noisy pooled mean in the denominator makes the estimate lean high)."""
    import torch

    from vk_cinematic_gb300.denoiser import KPCNN

    g = torch.Generator(device="cuda").manual_seed(21)
    B, H, W, tile = 1, 48, 64, 16
    sigma, spp_a, spp_c = 0.6, 4, 4
    mu = torch.full((B, H, W, 4), 1.0, device="cuda")
    A = mu + sigma / spp_a ** 0.5 * torch.randn((B, H, W, 4), device="cuda", generator=g)
    C = mu + sigma / spp_c ** 0.5 * torch.randn((B, H, W, 4), device="cuda", generator=g)
    D = mu.clone()
    D[0, 16:32, 32:48, :3] += 0.5
    net = KPCNN(seed=0)
    err, flags, need = net.check_tiles(D, A, spp_a, C, spp_c, bound=0.01, tile=tile, max_spp=4096,
                                       margin=2.0)
    torch.cuda.synchronize()
    f = flags.cpu().numpy().reshape(3, 4)
    bad = np.zeros((3, 4), bool)
    bad[1, 2] = True
    print("estimates", err.cpu().numpy().round(4).reshape(3, 4))
    print("need spp", need.cpu().numpy().reshape(3, 4))
    assert np.array_equal(f.astype(bool), bad)
    nd = need.cpu().numpy().astype(np.float64)
    expect = 2 * sigma ** 2 / 1.01 / 0.01
    assert np.all((nd > 0.85 * expect) & (nd < 1.6 * expect)), (nd, expect)
    assert expect <= nd.mean() <= 1.35 * expect, (nd.mean(), expect)
    # merge: flagged tile = weighted mean of the plain samples (and a fallback render)
    Fb = mu + 0.1 * torch.randn((B, H, W, 4), device="cuda", generator=g)
    spp_f = torch.zeros(12, dtype=torch.int32, device="cuda")
    spp_f[1 * 4 + 2] = 32
    out = net.merge_tiles(D, A, spp_a, C, spp_c, Fb, spp_f, flags, tile)
    torch.cuda.synchronize()
    exp = (spp_a * A + spp_c * C + 32 * Fb) / (spp_a + spp_c + 32)
    o = out.cpu()
    assert torch.allclose(o[0, 16:32, 32:48, :3], exp.cpu()[0, 16:32, 32:48, :3], rtol=1e-6,
                          atol=1e-6)
    keep = torch.ones((H, W), dtype=torch.bool)
    keep[16:32, 32:48] = False
    assert torch.equal(o[0][keep][:, :3], D.cpu()[0][keep][:, :3])


@pytest.mark.parametrize("check_spp", [None, 1])
def test_served_output_runs_end_to_end(gpu_lib, check_spp):
    """KPCNN.serve on a small scene: input render + G-buffers, denoise, check
    render (the input's spp, or 1), tile check, fallback tile-list renders,
    merge; the served image is finite and most tiles of an untrained network
    fall back."""
    import torch

    from vk_cinematic_gb300 import denoiser

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    rt = gbsp.Runtime(0, stream=stream.cuda_stream)
    s = scenes.config3_scene(width=160, height=96, spp=2, n_spheres=32, level=2, seed=8)
    sr = denoiser.SceneRenderer(rt, s)
    net = denoiser.KPCNN(seed=0)
    out, st = net.serve(sr, 0, 0, s.width, s.height, 2, seed=3, bound=0.01, check_spp=check_spp)
    torch.cuda.synchronize()
    print("served stats", {k: v for k, v in st.items() if k != "denoised"})
    assert out.shape == (s.height, s.width, 4)
    assert torch.isfinite(out).all()
    assert st["tiles"] == 6 * 10
    # an untrained network is far from the bound: most tiles fall back
    assert st["flagged"] > 0 and st["fallback_samples"] > 0
    torch.cuda.set_stream(torch.cuda.default_stream())
