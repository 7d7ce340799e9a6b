"""Test infrastructure only: a numpy FP32 restatement of the headless splat
(plg_render), the checker for the CUDA kernel.

It restates the app's default particle shaders
(resources/shaders/default.vert: the palette colour of the type;
default.geom:24-88: a square of side `size` around the centre minus
camTopLeft, wrapped with mod 1 and copied across the edges it is within
size/2 of; default.frag:7-12: discard where length(texCoord) > 1) under the
camera transform of utils/NormalizedDeviceCoordinates.java:42-48 and the
viewport transform, rasterised the way the library does it: 16 samples per
pixel on a 4x4 grid, the disk test once per pixel at its centre, the square
test per sample, the last particle in array order winning each sample
(opaque "normal" blending), then the average of the samples rounded to 8
bits.  Every operation is a single FP32 operation in the kernel's order, so
the image must match bit for bit.
"""
import numpy as np

F = np.float32
SAMPLES = 4  # per axis


def splat(pos, types, palette, width, height, cam=(0.5, 0.5, 1.0, 1.0), top_left=(0.0, 0.0), size=0.015,
          wrap=False):
    """(height, width, 4) uint8, rows bottom to top.  pos: (n, >=2) float32
    in draw order; palette: (k, 4) float32 RGBA."""
    pos = np.asarray(pos, np.float32)
    pal = np.asarray(palette, np.float32).reshape(-1, 4)
    cam_x, cam_y, cam_w, cam_h = (F(c) for c in cam)
    tl_x, tl_y = F(top_left[0]), F(top_left[1])
    size = F(size)
    winner = np.zeros((height, width, SAMPLES, SAMPLES), np.int64)
    sub = (np.arange(SAMPLES, dtype=np.float32) + F(0.5)) / F(SAMPLES)
    r = F(0.5) * size
    sx = F(width) / cam_w
    sy = F(height) / cam_h
    hw, hh = F(0.5) * F(width), F(0.5) * F(height)

    def one(cx, cy, tag):
        px0 = ((cx - r) - cam_x) * sx + hw
        px1 = ((cx + r) - cam_x) * sx + hw
        py0 = ((cy - r) - cam_y) * sy + hh
        py1 = ((cy + r) - cam_y) * sy + hh
        pcx = (cx - cam_x) * sx + hw
        pcy = (cy - cam_y) * sy + hh
        rpx, rpy = r * sx, r * sy
        if not all(np.isfinite(v) for v in (px0, px1, py0, py1)):
            return
        i0, i1 = int(max(np.floor(px0), 0)), int(min(np.floor(px1), width - 1))
        j0, j1 = int(max(np.floor(py0), 0)), int(min(np.floor(py1), height - 1))
        if i0 > i1 or j0 > j1:
            return
        ii = np.arange(i0, i1 + 1, dtype=np.float32)
        jj = np.arange(j0, j1 + 1, dtype=np.float32)
        tx = ((ii + F(0.5)) - pcx) / rpx
        ty = ((jj + F(0.5)) - pcy) / rpy
        disk = np.sqrt(ty[:, None] * ty[:, None] + tx[None, :] * tx[None, :]) <= F(1)
        xx = ii[:, None] + sub[None, :]  # (pixels x, samples a)
        yy = jj[:, None] + sub[None, :]
        inx = (xx >= px0) & (xx < px1)
        iny = (yy >= py0) & (yy < py1)
        m = disk[:, :, None, None] & iny[:, None, :, None] & inx[None, :, None, :]
        blk = winner[j0:j1 + 1, i0:i1 + 1]
        blk[m] = tag

    for k in range(pos.shape[0]):
        cx, cy = pos[k, 0] - tl_x, pos[k, 1] - tl_y
        if wrap:
            cx, cy = cx - np.floor(cx), cy - np.floor(cy)
        one(cx, cy, k + 1)
        if wrap:
            dx = 1 if cx < r else (-1 if cx > F(1) - r else 0)
            dy = 1 if cy < r else (-1 if cy > F(1) - r else 0)
            if dx:
                one(cx + F(dx), cy, k + 1)
            if dy:
                one(cx, cy + F(dy), k + 1)
            if dx and dy:
                one(cx + F(dx), cy + F(dy), k + 1)

    t = np.asarray(types, np.int64)
    w = winner.reshape(height, width, SAMPLES * SAMPLES)
    acc = np.zeros((height, width, 4), np.float32)
    for s in range(SAMPLES * SAMPLES if len(t) else 0):  # sample order, as the resolve adds them
        ws = w[:, :, s]
        hit = ws > 0
        ty = np.minimum(t[np.maximum(ws - 1, 0)], pal.shape[0] - 1)
        acc = np.where(hit[:, :, None], acc + pal[ty], acc)
    v = acc * F(1.0 / (SAMPLES * SAMPLES))
    return np.rint(np.clip(v, F(0), F(1)) * F(255)).astype(np.uint8)
