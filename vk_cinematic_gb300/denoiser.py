"""Kernel-predicting CNN denoiser on libgbsp's denoiser kernels.

Network (the config-5 description): 8 conv3x3 layers, 10 -> 48, six 48 -> 48,
48 -> 25, ReLU between layers; the 25 outputs of a pixel are softmax weights
of a 5x5 filter applied to the noisy radiance around it.  Inputs: log(1 +
radiance), albedo, normal and depth/(1 + depth) of a low-spp frame, BF16.
Training minimises relMSE = mean((out - ref)^2 / (ref^2 + 0.01)) with Adam.

Every arithmetic step runs in libgbsp kernels (include/gbsp.h,
"learned denoiser"); torch only provides device memory and the stream.
"""

from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from . import gbsp, scenes

N_FEATURES = 10
FEATURE_CHANNELS = 16
# (cin, cout, epilogue): epilogue 0 = BF16 ReLU, 1 = FP32 logits
LAYERS = [(16, 48, 0)] + [(48, 48, 0)] * 6 + [(48, 32, 1)]

_c = ctypes
_u32, _u64, _f32, _int, _vp = _c.c_uint32, _c.c_uint64, _c.c_float, _c.c_int, _c.c_void_p


def _stream():
    import torch

    return _vp(torch.cuda.current_stream().cuda_stream)


def _ptr(t) -> _vp:
    return _vp(t.data_ptr())


def _check(rc):
    gbsp._check(rc)


def to_planar(t):
    """NHWC (B, H, W, C) -> the kernels' channel-group-planar (B, H, C/8, W, 8)."""
    B, H, W, C = t.shape
    return t.reshape(B, H, W, C // 8, 8).permute(0, 1, 3, 2, 4).contiguous()


def from_planar(t):
    """Channel-group-planar (B, H, C/8, W, 8) -> NHWC (B, H, W, C)."""
    B, H, G, W, _ = t.shape
    return t.permute(0, 1, 3, 2, 4).reshape(B, H, W, G * 8)


def _dims(t):
    """(B, H, W, C) of a channel-group-planar activation tensor."""
    B, H, G, W, _ = t.shape
    return B, H, W, G * 8


def relmse(x, ref):
    """mean over pixels and RGB of (x - ref)^2 / (ref^2 + 0.01)."""
    import torch

    x = x[..., :3].double()
    r = ref[..., :3].double()
    return float(torch.mean((x - r) ** 2 / (r * r + 0.01)).item())


class KPCNN:
    """conv: "tcgen05" (5th-generation tensor cores, accumulator in tensor
    memory) or "mma" (mma.sync BF16 fragments) for the forward and
    data-gradient convolutions.  wgrad: "tcgen05" (5th-generation tensor
    cores, operands loaded by TMA, accumulators in tensor memory), "mma"
    (mma.sync fragments) - both with deterministic per-CTA partial sums - or
    "simt" (FP32 FMA with atomics) for the weight gradient."""

    def __init__(self, seed: int = 0, conv: str = "tcgen05", wgrad: str = "tcgen05"):
        import torch

        self.L = gbsp.load()
        self._conv = {"tcgen05": self.L.gbsp_dn_conv3x3_forward_tc,
                      "mma": self.L.gbsp_dn_conv3x3_forward}[conv]
        self._wgrad = {"tcgen05": self.L.gbsp_dn_conv3x3_weight_grad_tcgen05,
                       "mma": self.L.gbsp_dn_conv3x3_weight_grad_tc,
                       "simt": self.L.gbsp_dn_conv3x3_weight_grad}[wgrad]
        self.conv_impl = conv
        self.wgrad_impl = wgrad
        g = torch.Generator().manual_seed(seed)
        self.w, self.b, self.wb, self.state = [], [], [], []
        for li, (cin, cout, epi) in enumerate(LAYERS):
            fan_in = 9 * (N_FEATURES if cin == FEATURE_CHANNELS else cin)
            std = math.sqrt(2.0 / fan_in) * (0.1 if epi == 1 else 1.0)
            w = torch.randn((9, cout, cin), generator=g) * std
            if cin == FEATURE_CHANNELS:
                w[:, :, N_FEATURES:] = 0
            if epi == 1:
                w[:, 25:, :] = 0
            w = w.cuda().contiguous()
            b = torch.zeros(cout, device="cuda")
            self.w.append(w)
            self.b.append(b)
            self.wb.append(w.to(torch.bfloat16).contiguous())
            self.state.append([torch.zeros_like(w), torch.zeros_like(w), torch.zeros_like(b),
                               torch.zeros_like(b)])
        self.step = 0

    def parameters_count(self) -> int:
        return sum(w.numel() + b.numel() for w, b in zip(self.w, self.b))

    # ---- forward -----------------------------------------------------------------
    def features(self, radiance, aov):
        import torch

        B, H, W, _ = radiance.shape
        f = torch.empty((B, H, FEATURE_CHANNELS // 8, W, 8), dtype=torch.bfloat16, device="cuda")
        _check(self.L.gbsp_dn_features(_stream(), _ptr(radiance), _ptr(aov), _u64(B * H * W),
                                       _u32(W), _ptr(f)))
        return f

    def conv(self, li, x, keep_f32=False):
        import torch

        B, H, W, cin = _dims(x)
        _, cout, _ = self.wb[li].shape
        epi = LAYERS[li][2]
        if epi == 0:
            out = torch.empty((B, H, cout // 8, W, 8), dtype=torch.bfloat16, device="cuda")
            _check(self._conv(_stream(), _ptr(x), _u32(B), _u32(H), _u32(W), _u32(cin),
                              _ptr(self.wb[li]), _ptr(self.b[li]), _u32(cout), _int(0), _ptr(out),
                              None))
        else:
            out = torch.empty((B, H, W, cout), dtype=torch.float32, device="cuda")
            _check(self._conv(_stream(), _ptr(x), _u32(B), _u32(H), _u32(W), _u32(cin),
                              _ptr(self.wb[li]), _ptr(self.b[li]), _u32(cout), _int(1), None,
                              _ptr(out)))
        return out

    def forward(self, feats, keep=False):
        acts = []
        x = feats
        for li in range(len(LAYERS)):
            x = self.conv(li, x)
            if keep and li < len(LAYERS) - 1:
                acts.append(x)
        return x, acts

    def filter(self, logits, noisy):
        import torch

        B, H, W, _ = noisy.shape
        out = torch.empty_like(noisy)
        _check(self.L.gbsp_dn_filter(_stream(), _ptr(logits), _ptr(noisy), _u32(B), _u32(H),
                                     _u32(W), _ptr(out)))
        return out

    def denoise(self, radiance, aov):
        """Denoised RGBA32F frame.  On the tcgen05 path the logits layer and the
        5x5 filter run as one kernel (the logits never reach memory); the
        result is bit-identical to forward() + filter()."""
        import torch

        if self.conv_impl != "tcgen05":
            logits, _ = self.forward(self.features(radiance, aov))
            return self.filter(logits, radiance)
        x = self.features(radiance, aov)
        last = len(LAYERS) - 1
        for li in range(last):
            x = self.conv(li, x)
        B, H, W, cin = _dims(x)
        noisy = radiance.contiguous()
        out = torch.empty((B, H, W, 4), dtype=torch.float32, device="cuda")
        _check(self.L.gbsp_dn_conv3x3_filter_tc(_stream(), _ptr(x), _u32(B), _u32(H), _u32(W),
                                                _u32(cin), _ptr(self.wb[last]), _ptr(self.b[last]),
                                                _ptr(noisy), _ptr(out)))
        return out

    def denoise_checked(self, radiance, aov, plain_check, bound=0.01, tile=16):
        """Denoises `radiance` and lets the plain path tracer check every
        tile x tile block with an independent render `plain_check` of the same
        spp (gbsp_dn_tile_fallback): blocks whose estimated relMSE exceeds
        `bound` by more than two standard errors are served from the plain
        samples.  Returns (image, per-tile estimates, per-tile fallback
        flags)."""
        import torch

        den = self.denoise(radiance, aov)
        B, H, W, _ = radiance.shape
        tiles = B * ((H + tile - 1) // tile) * ((W + tile - 1) // tile)
        out = torch.empty_like(den)
        err = torch.empty(tiles, dtype=torch.float32, device="cuda")
        flags = torch.empty(tiles, dtype=torch.int32, device="cuda")
        _check(self.L.gbsp_dn_tile_fallback(_stream(), _ptr(den), _ptr(radiance),
                                            _ptr(plain_check), _u32(B), _u32(H), _u32(W),
                                            _u32(tile), _f32(bound), _ptr(out), _ptr(err),
                                            _ptr(flags)))
        return out, err, flags

    def check_tiles(self, denoised, plain_a, spp_a, plain_c, spp_c, bound=0.01, tile=16,
                    max_spp=4096, margin=1.25):
        """gbsp_dn_tile_check: per tile x tile block, the estimated relMSE of the
        denoised frames, the flag (estimate above `bound` by two standard
        errors) and the plain spp that brings the tile to `bound`."""
        import torch

        B, H, W, _ = denoised.shape
        tiles = B * ((H + tile - 1) // tile) * ((W + tile - 1) // tile)
        err = torch.empty(tiles, dtype=torch.float32, device="cuda")
        flags = torch.empty(tiles, dtype=torch.int32, device="cuda")
        need = torch.empty(tiles, dtype=torch.int32, device="cuda")
        _check(self.L.gbsp_dn_tile_check(_stream(), _ptr(denoised), _ptr(plain_a), _u32(spp_a),
                                         _ptr(plain_c), _u32(spp_c), _u32(B), _u32(H), _u32(W),
                                         _u32(tile), _f32(bound), _f32(margin), _u32(max_spp),
                                         _ptr(err), _ptr(flags), _ptr(need)))
        return err, flags, need

    def merge_tiles(self, denoised, plain_a, spp_a, plain_c, spp_c, fallback, spp_f, flags,
                    tile=16):
        """gbsp_dn_tile_merge: the served frames."""
        import torch

        B, H, W, _ = denoised.shape
        out = torch.empty_like(denoised)
        _check(self.L.gbsp_dn_tile_merge(_stream(), _ptr(denoised), _ptr(plain_a), _u32(spp_a),
                                         _ptr(plain_c), _u32(spp_c),
                                         _ptr(fallback) if fallback is not None else None,
                                         _ptr(spp_f) if spp_f is not None else None, _u32(B),
                                         _u32(H), _u32(W), _u32(tile), _ptr(flags), _ptr(out)))
        return out

    def serve(self, sr, x0, y0, w, h, spp, seed, bound=0.01, tile=16, max_spp=1024, margin=1.25,
              timing=None, check_spp=None):
        """The served output of a w x h window of `sr`'s frame: `spp`-sample plain
        render + G-buffers -> denoised; an independent `check_spp`-sample plain
        render (default `spp`; the next samples of the same per-pixel sequence,
        rendered in the same pass as the input) checks every tile x tile block
        (check_tiles); blocks that fail are served from all their plain samples,
        topped up by a
        fallback render to the spp the check estimated for `bound` (every
        flagged block in one tile-list pass, each at its own sample count).
        Returns (image, stats): stats counts the flagged blocks and the fallback
        samples rendered, and holds the unchecked denoised image under
        "denoised"."""
        import torch

        cspp = spp if check_spp is None else int(check_spp)
        ev = [] if timing is not None else None

        def mark():
            if ev is not None:
                e = torch.cuda.Event(enable_timing=True)
                e.record()
                ev.append(e)

        mark()
        # input (samples 0 .. spp - 1, with G-buffers) and the independent check
        # render (samples spp .. spp + cspp - 1 of the same per-pixel sequence) in
        # one pass
        rad, aov, chk = sr.render_split(x0, y0, w, h, spp, cspp, seed, aov=True)
        mark()
        den = self.denoise(rad.unsqueeze(0).contiguous(), aov.unsqueeze(0).contiguous())
        mark()
        err, flags, need = self.check_tiles(den, rad.unsqueeze(0).contiguous(), spp,
                                            chk.unsqueeze(0).contiguous(), cspp, bound, tile,
                                            max_spp, margin)
        f = flags.cpu().numpy()
        nd = need.cpu().numpy().astype(np.int64)
        tx = (w + tile - 1) // tile
        # flagged tiles that need samples beyond the two plain renders
        extra = np.where(f != 0, nd - spp - cspp, 0)
        sel = np.nonzero(extra > 0)[0]
        spp_f = np.zeros(len(f), np.int32)
        spp_f[sel] = extra[sel]
        bx, by = (sel % tx) * tile, (sel // tx) * tile
        fb_tiles = np.stack([x0 + bx, y0 + by, x0 + np.minimum(bx + tile, w),
                             y0 + np.minimum(by + tile, h)], axis=1).astype(np.uint32)
        fb_spp = extra[sel].astype(np.uint32)
        mark()
        fb = None
        fb_samples = 0
        if len(sel):
            sr.render_tiles_spp(fb_tiles, fb_spp, (seed + 7919) & 0xFFFFFFFF)
            area = (fb_tiles[:, 2].astype(np.int64) - fb_tiles[:, 0]) * (fb_tiles[:, 3].astype(np.int64) - fb_tiles[:, 1])
            fb_samples = int((fb_spp.astype(np.int64) * area).sum())
            fb = torch.empty((1, h, w, 4), dtype=torch.float32, device="cuda")
            sr.rend.copy_region(x0, y0, w, h, fb.data_ptr())
        mark()
        out = self.merge_tiles(den, rad.unsqueeze(0).contiguous(), spp,
                               chk.unsqueeze(0).contiguous(), cspp, fb,
                               torch.from_numpy(spp_f).cuda() if fb is not None else None, flags,
                               tile)
        mark()
        if ev is not None:
            torch.cuda.synchronize()
            names = ["input_and_check_render", "denoise", "check_and_readback",
                     "fallback_renders", "merge"]
            for k, n in enumerate(names):
                timing[n] = timing.get(n, 0.0) + ev[k].elapsed_time(ev[k + 1])
        stats = {"tiles": int(len(f)), "flagged": int(f.sum()), "fallback_samples": fb_samples,
                 "fallback_tiles": int(len(sel)), "denoised": den[0]}
        return out[0], stats

    # ---- training ------------------------------------------------------------------
    def data_grad(self, li, d):
        """dIn of layer li from its output gradient d (BF16), FP32; both
        channel-group-planar."""
        import torch

        B, H, W, cout = _dims(d)
        _, _, cin = self.wb[li].shape
        wt = torch.empty((9, cin, cout), dtype=torch.bfloat16, device="cuda")
        _check(self.L.gbsp_dn_flip_transpose(_stream(), _ptr(self.wb[li]), _u32(cout), _u32(cin),
                                             _ptr(wt)))
        out = torch.empty((B, H, cin // 8, W, 8), dtype=torch.float32, device="cuda")
        _check(self._conv(_stream(), _ptr(d), _u32(B), _u32(H), _u32(W), _u32(cout), _ptr(wt),
                          None, _u32(cin), _int(2), None, _ptr(out)))
        return out

    def weight_grad(self, li, x, d, dw, db):
        B, H, W, cin = _dims(x)
        cout = _dims(d)[3]
        _check(self._wgrad(_stream(), _ptr(x), _ptr(d), _u32(B), _u32(H), _u32(W), _u32(cin),
                           _u32(cout), _ptr(dw), _ptr(db)))

    def gradients(self, feats, noisy, target):
        """Loss and parameter gradients for one batch."""
        import torch

        B, H, W, _ = noisy.shape
        logits, acts = self.forward(feats, keep=True)
        dlog = torch.empty((B, H, 4, W, 8), dtype=torch.bfloat16, device="cuda")
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        _check(self.L.gbsp_dn_relmse_backward(_stream(), _ptr(logits), _ptr(noisy), _ptr(target),
                                              _u32(B), _u32(H), _u32(W), _ptr(dlog), _ptr(loss)))
        dws = [torch.zeros_like(w) for w in self.w]
        dbs = [torch.zeros_like(b) for b in self.b]
        last = len(LAYERS) - 1
        inputs = [feats] + acts
        self.weight_grad(last, inputs[last], dlog, dws[last], dbs[last])
        dact = self.data_grad(last, dlog)
        for li in range(last - 1, -1, -1):
            dm = torch.empty(acts[li].shape, dtype=torch.bfloat16, device="cuda")
            _check(self.L.gbsp_dn_relu_backward(_stream(), _ptr(dact), _ptr(acts[li]),
                                                _u64(dact.numel()), _ptr(dm)))
            self.weight_grad(li, inputs[li], dm, dws[li], dbs[li])
            if li > 0:
                dact = self.data_grad(li, dm)
        return loss, dws, dbs

    def train_step(self, feats, noisy, target, lr=1e-4):
        loss, dws, dbs = self.gradients(feats, noisy, target)
        self.step += 1
        for li in range(len(LAYERS)):
            m, v, mb, vb = self.state[li]
            _check(self.L.gbsp_dn_adam(_stream(), _ptr(self.w[li]), _ptr(self.wb[li]),
                                       _ptr(dws[li]), _ptr(m), _ptr(v), _u64(self.w[li].numel()),
                                       _f32(lr), _f32(0.9), _f32(0.999), _f32(1e-8),
                                       _u32(self.step)))
            _check(self.L.gbsp_dn_adam(_stream(), _ptr(self.b[li]), None, _ptr(dbs[li]),
                                       _ptr(mb), _ptr(vb), _u64(self.b[li].numel()), _f32(lr),
                                       _f32(0.9), _f32(0.999), _f32(1e-8), _u32(self.step)))
        B, H, W, _ = noisy.shape
        return loss / (3.0 * B * H * W)


# ---- data from the path tracer --------------------------------------------------------
def denoise_scene(seed, width=1920, height=1080, n_spheres=256, level=5):
    """A config-3-style scene (the config-5 scene family)."""
    return scenes.config3_scene(width=width, height=height, spp=4, max_bounces=5,
                                n_spheres=n_spheres, level=level, seed=seed)


class SceneRenderer:
    """One uploaded scene that renders windows at any spp and seed."""

    def __init__(self, rt, s):
        self.s = s
        self.scene, self.ms, self.rend = gbsp.upload_scene(rt, s)
        self._image2 = None  # second image of split renders (full frame)

    def render(self, x0, y0, w, h, spp, seed, aov=False):
        import torch

        o = self.rend.options
        o.spp, o.seed = spp, seed
        o.flags = gbsp.FLAG_AOV if aov else 0
        self.rend.tile_device((x0, y0, x0 + w, y0 + h))
        rad = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
        av = torch.empty((h, w, 8), dtype=torch.float32, device="cuda") if aov else None
        self.rend.copy_region(x0, y0, w, h, rad.data_ptr(), av.data_ptr() if aov else 0)
        return rad, av

    def render_split(self, x0, y0, w, h, spp_a, spp_c, seed, aov=True):
        """One pass of spp_a + spp_c samples per pixel over the window: returns
        the mean of the first spp_a (the image a spp_a render gives, with its
        G-buffers) and the mean of the other spp_c, an independent render."""
        import torch

        o = self.rend.options
        o.spp, o.seed = spp_a + spp_c, seed
        o.flags = gbsp.FLAG_AOV if aov else 0
        if self._image2 is None:
            self._image2 = torch.empty((self.s.height, self.s.width, 4), dtype=torch.float32,
                                       device="cuda")
        self.rend.tile_split_device((x0, y0, x0 + w, y0 + h), spp_a, self._image2.data_ptr())
        rad = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
        av = torch.empty((h, w, 8), dtype=torch.float32, device="cuda") if aov else None
        self.rend.copy_region(x0, y0, w, h, rad.data_ptr(), av.data_ptr() if aov else 0)
        chk = self._image2[y0:y0 + h, x0:x0 + w].contiguous()
        return rad, av, chk

    def render_tiles(self, tiles, spp, seed):
        """Plain render of the listed (minX, minY, maxX, maxY) frame tiles at
        `spp` in one pass, into the runtime's frame buffer."""
        o = self.rend.options
        o.spp, o.seed = spp, seed
        o.flags = 0
        self.rend.tile_list_device(tiles)

    def render_tiles_spp(self, tiles, spp, seed):
        """Plain render of the listed (minX, minY, maxX, maxY) frame tiles, tile
        i at spp[i], in one pass into the runtime's frame buffer."""
        o = self.rend.options
        o.seed = seed
        o.flags = 0
        self.rend.tile_list_spp_device(tiles, spp)

    def reference(self, x0, y0, w, h, spp_total, per_pass=1024, seed=1 << 20):
        """FP64-accumulated high-spp image: the mean of FP32 passes, summed in FP64."""
        import torch

        passes = max(1, spp_total // per_pass)
        acc = torch.zeros((h, w, 4), dtype=torch.float64, device="cuda")
        for k in range(passes):
            rad, _ = self.render(x0, y0, w, h, min(per_pass, spp_total), seed + k)
            acc += rad.double()
        return (acc / passes)


def make_dataset(rt, n_scenes, crops_per_scene, crop=128, spp_in=4, spp_ref=4096, seed0=0,
                 n_spheres=256, level=5, log=print):
    """Training pairs: random crops of config-3-style frames, low-spp inputs
    (+ G-buffers) and independent high-spp targets.  spp_in may be a sequence:
    crop c then gets spp_in[c % len(spp_in)] samples (a mixed-noise dataset)."""
    import torch

    spp_list = list(spp_in) if isinstance(spp_in, (list, tuple)) else [spp_in]
    rng = np.random.default_rng(seed0)
    feats_l, noisy_l, tgt_l = [], [], []
    t0 = time.time()
    for k in range(n_scenes):
        s = denoise_scene(seed0 + k, n_spheres=n_spheres, level=level)
        sr = SceneRenderer(rt, s)
        for c in range(crops_per_scene):
            x0 = int(rng.integers(0, s.width - crop))
            y0 = int(rng.integers(0, s.height - crop))
            spp = spp_list[c % len(spp_list)]
            noisy, aov = sr.render(x0, y0, crop, crop, spp, seed=1000 * k + 2 * c, aov=True)
            target, _ = sr.render(x0, y0, crop, crop, spp_ref, seed=1000 * k + 2 * c + 1)
            noisy_l.append(noisy)
            tgt_l.append(target)
            feats_l.append(aov)
    torch.cuda.synchronize()
    log(f"dataset: {len(noisy_l)} crops in {time.time() - t0:.1f} s")
    return torch.stack(noisy_l), torch.stack(feats_l), torch.stack(tgt_l)
