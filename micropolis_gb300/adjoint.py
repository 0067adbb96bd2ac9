"""Differentiable rendering: image-loss gradients with respect to control
points and the displacement amplitude, visibility held fixed.

RenderFunction.forward renders through the C ABI (batched path) and keeps the
frame's per-pixel winning micropolygon; backward runs the hand-written
adjoint kernel (mp_backward), which recomputes the winning quads' dice
vertices instead of storing grids.  PyTorch is used for tensors and streams
only.
"""
from __future__ import annotations

import torch

from .renderer import Projection, Renderer, renderer_for


class DiffRenderer:
    """A renderer bound to one mesh (draw 0, view 0) for gradient work."""

    def __init__(self, scene, handle: int = 1):
        d = scene.draws[0]
        self.scene = scene
        self.draw = d
        self.handle = handle
        self.n_patches = d.mesh.n_patches
        self.per = d.mesh.cp.shape[1]
        self.r: Renderer = renderer_for(scene, "batched")
        self.proj = Projection(scene.fovy, scene.near, (scene.width, scene.height))
        self.r.load_patches(handle, d.mesh.cp, d.mesh.type)
        self.npx = scene.width * scene.height
        self._side = None

    def _stream_in(self):
        """Binds the renderer to the stream of a call made on torch's
        current stream: that stream itself, or -- for the legacy default
        stream, on which a frame's CUDA graph cannot be captured -- a side
        stream that first waits for it.  Returns (caller's stream, side
        stream or None) for _stream_out."""
        cur = torch.cuda.current_stream()
        if cur.cuda_stream != 0:
            self.r.set_stream(cur.cuda_stream)
            return cur, None
        if self._side is None:
            self._side = torch.cuda.Stream(device=cur.device)
        self._side.wait_stream(cur)
        self.r.set_stream(self._side.cuda_stream)
        return cur, self._side

    @staticmethod
    def _stream_out(cur, side, *tensors):
        """The caller's stream waits for the side stream's work on `tensors`."""
        if side is not None:
            for t in tensors:
                t.record_stream(side)
            cur.wait_stream(side)

    def render(self, cp: torch.Tensor, amp) -> torch.Tensor:
        """Tiled RGBA image (W*H, 4) for control points cp (n, per, 3) and
        the displacement amplitude multiplier amp: a tensor on the device
        (read there, no host synchronization) or a number."""
        xyz1 = torch.cat([cp.detach().float().reshape(-1, 3),
                          torch.ones(cp.numel() // 3, 1, device=cp.device)], dim=1).contiguous()
        amp_dev = None
        if isinstance(amp, torch.Tensor):
            amp_dev = amp.detach().to(device=cp.device, dtype=torch.float32).reshape(1).contiguous()
        img = torch.empty((self.npx, 4), dtype=torch.float32, device=cp.device)
        cur, side = self._stream_in()
        self.r.update_patches_device(self.handle, xyz1.data_ptr())
        if amp_dev is not None:
            self.r.set_displacement_amplitude_device(amp_dev.data_ptr())
        else:
            self.r.set_displacement_amplitude(float(amp))
        self.r.prepare()
        self.r.draw_patches(self.handle, self.draw.mv, self.proj, self.draw.color)
        self.r.finish()
        self.r.copy_framebuffer_device(0, img.data_ptr())
        self._stream_out(cur, side, img, xyz1, *([amp_dev] if amp_dev is not None else []))
        return img

    def backward(self, grad_img: torch.Tensor, cp_shape, device):
        n = 1
        for k in cp_shape:
            n *= int(k)
        g_cp = torch.zeros(n, dtype=torch.float32, device=device)
        g_amp = torch.zeros(1, dtype=torch.float32, device=device)
        g_img = grad_img.contiguous()
        cur, side = self._stream_in()
        self.r.set_grad_buffer(0, g_cp.data_ptr())
        self.r.backward(0, g_img.data_ptr(), g_amp.data_ptr())
        self._stream_out(cur, side, g_cp, g_amp, g_img)
        return g_cp.reshape(cp_shape), g_amp


class RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, cp: torch.Tensor, amp: torch.Tensor, dr: DiffRenderer):
        img = dr.render(cp, amp)
        ctx.dr = dr
        ctx.cp_shape = tuple(cp.shape)
        ctx.device = cp.device
        return img

    @staticmethod
    def backward(ctx, grad_img):
        g_cp, g_amp = ctx.dr.backward(grad_img, ctx.cp_shape, ctx.device)
        return g_cp, g_amp.reshape(()), None


def render(cp: torch.Tensor, amp: torch.Tensor, dr: DiffRenderer) -> torch.Tensor:
    return RenderFunction.apply(cp, amp, dr)


def bench_bwd_fwd(stream=None, steps: int = 10, workload: str = "heightfield16_512x512") -> dict:
    """Forward (frame) and backward (adjoint) device times on a displaced
    heightfield workload (default the 16x16 one at 512x512) with an L2 image
    loss against a target rendered from perturbed control points: N(0, 0.05)
    for 16 x 16 patches, scaled with the patch spacing for finer grids.  Runs
    on `stream` (a torch stream; None: the current stream), with CUDA events
    on that stream around the autograd forward and the backward."""
    import contextlib
    import numpy as np
    from . import scenes
    ctx = torch.cuda.stream(stream) if stream is not None else contextlib.nullcontext()
    with ctx:
        return _bench_bwd_fwd(steps, workload, np, scenes)


def _bench_bwd_fwd(steps, workload, np, scenes) -> dict:
    sc = scenes.WORKLOADS[workload]()
    dev = torch.device("cuda")
    dr = DiffRenderer(sc)
    cp0 = torch.tensor(sc.draws[0].mesh.cp, device=dev)
    rng = np.random.default_rng(sc.seed + 100)
    sigma = 0.05 * 16.0 / max(16.0, float(np.sqrt(sc.n_patches)))
    cpt = cp0 + torch.tensor(rng.normal(0, sigma, size=cp0.shape).astype(np.float32), device=dev)
    target = dr.render(cpt, 1.2).clone()
    cp = cp0.clone().requires_grad_(True)
    amp = torch.tensor(1.0, device=dev, requires_grad=True)
    fwd, bwd, frame = [], [], []
    for i in range(steps + 3):
        a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        a.record()
        img = render(cp, amp, dr)
        b.record()
        loss = ((img - target) ** 2).sum()
        g = 2 * (img - target)
        b2 = torch.cuda.Event(enable_timing=True)
        b2.record()
        g_cp, g_amp = dr.backward(g, tuple(cp.shape), dev)
        c.record()
        torch.cuda.synchronize()
        if i >= 3:
            fwd.append(a.elapsed_time(b))
            bwd.append(b2.elapsed_time(c))
            frame.append(dr.r.stats()["gpu_ms"])
        del loss
    f, bk, fr = float(np.median(fwd)), float(np.median(bwd)), float(np.median(frame))
    work = backward_work(sc, dr.r)
    # fwd_ms: the autograd forward as a caller sees it (control-point
    # widening and upload, amplitude copy, the frame, the image copy);
    # frame_ms: the batched frame alone (device time of its graph)
    return {"workload": f"{workload} (displacement on)", "fwd_ms": f, "frame_ms": fr, "bwd_ms": bk,
            "bwd_over_fwd": bk / f, "bwd_over_frame": bk / fr, **work,
            "bwd_gbs": work["B_bwd"] / (bk / 1e3) / 1e9, "bwd_updates_per_s": work["A_bwd"] / (bk / 1e3)}


def backward_work(scene, r, view: int = 0) -> dict:
    """Algorithmic work of one backward pass over the last frame of r:
    B_bwd = W*H*(8 + 16 + 16) B (the depth|id key, dL/dcolour and the
    colour of every pixel) + 12 B per control point of the gradient;
    A_bwd = control-point gradient updates the adjoint kernel issues (one
    per control-point coordinate per warp of 32 pixels when every pixel of
    the warp has the same winning patch, else one per covered pixel;
    updates of zero are skipped on the device, so this is an upper bound)."""
    import numpy as np
    W, H = scene.width, scene.height
    ncp = sum(d.mesh.n_patches * d.mesh.cp.shape[1] for d in scene.draws)
    vis = r.visibility(view)
    draw, pid, _ = r.subpatches()
    PS2 = r.options.reyes_patch_size ** 2
    covered = vis >= 0
    owner = np.full(len(vis), -1, np.int64)
    s = vis[covered] // PS2
    owner[covered] = (draw[s].astype(np.int64) << 32) | pid[s].astype(np.int64)
    per = np.zeros(len(vis), np.int64)
    cps = np.array([d.mesh.cp.shape[1] for d in scene.draws])
    per[covered] = cps[draw[s]] * 3
    n = len(vis) // 32 * 32
    wo = owner[:n].reshape(-1, 32)
    uniform = np.all(wo == wo[:, :1], axis=1) & (wo[:, 0] >= 0)
    a = int(per[:n].reshape(-1, 32)[~uniform].sum() + per[:n].reshape(-1, 32)[uniform, 0].sum() + per[n:].sum())
    return {"B_bwd": W * H * 40 + 12 * ncp, "A_bwd": a, "covered_pixels": int(covered.sum())}
