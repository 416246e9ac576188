"""Seeded synthetic frames for the JPEG XS encode/decode workloads.

Content model (one plane): a smooth 2-D linear gradient, Gaussian noise and
axis-aligned rectangles with uniform random fill (hard edges), clipped to the
sample range and rounded.  8-bit planes use the gradient range [16, 235] and
sigma 4; other depths rescale the 8-bit model by (2^d - 1) / 255 unless an
explicit range and sigma are given (the 4K 10-bit stream uses [64, 940] and
sigma 16).  Rectangles may drift by `drift` pixels per frame index.

Chroma planes of subsampled formats are built the same way at their own size.
"""
import numpy as np

# Colour format ids, equal to the ColourFormat_t values of the public API.
FMT_YUV400 = 1
FMT_YUV420 = 2
FMT_YUV422 = 3
FMT_YUV444 = 4
FMT_4COMP = 5
FMT_GRAY = 6
FMT_PACKED_RGB = 21


def component_dims(width, height, fmt):
    """(w, h) per component, following the sampling factors of each format."""
    if fmt == FMT_YUV422:
        return [(width, height), (width // 2, height), (width // 2, height)]
    if fmt == FMT_YUV420:
        return [(width, height), (width // 2, height // 2), (width // 2, height // 2)]
    if fmt in (FMT_YUV444, FMT_PACKED_RGB):
        return [(width, height)] * 3
    if fmt == FMT_4COMP:
        return [(width, height)] * 4
    if fmt in (FMT_GRAY, FMT_YUV400):
        return [(width, height)]
    raise ValueError("unsupported format %r" % fmt)


def plane(rng, w, h, depth, frame_idx=0, lo=None, hi=None, sigma=None, rects=20, drift=0, noise_quadrant=False):
    maxv = (1 << depth) - 1
    scale = maxv / 255.0
    if lo is None:
        lo = 16 * scale
    if hi is None:
        hi = 235 * scale
    if sigma is None:
        sigma = 4 * scale
    x = np.arange(w, dtype=np.float64) / max(w - 1, 1)
    y = np.arange(h, dtype=np.float64) / max(h - 1, 1)
    img = lo + (hi - lo) * (x[None, :] + y[:, None]) / 2.0
    img = img + rng.normal(0.0, sigma, size=(h, w))
    for _ in range(rects):
        x0, x1 = np.sort(rng.integers(0, w, size=2))
        y0, y1 = np.sort(rng.integers(0, h, size=2))
        val = rng.uniform(0, maxv)
        d = drift * frame_idx
        xa, xb = min(w, x0 + d), min(w, x1 + 1 + d)
        img[y0:y1 + 1, xa:xb] = val
    if noise_quadrant:
        img[: h // 2, : w // 2] = rng.integers(0, maxv + 1, size=(h // 2, w // 2))
    img = np.clip(np.rint(img), 0, maxv)
    return img.astype(np.uint8 if depth <= 8 else np.uint16)


def frame(width, height, depth, fmt, seed=0, frame_idx=0, lo=None, hi=None, sigma=None, drift=0, noise_quadrant=False):
    """Planes of one frame (list of 2-D arrays); packed RGB returns one (h, 3w) array."""
    rng = np.random.default_rng(seed)
    dims = component_dims(width, height, fmt)
    planes = [plane(rng, w, h, depth, frame_idx, lo, hi, sigma, drift=drift, noise_quadrant=noise_quadrant) for (w, h) in dims]
    if fmt == FMT_PACKED_RGB:
        packed = np.stack(planes, axis=-1).reshape(height, width * 3)
        return [np.ascontiguousarray(packed)]
    return planes


def frame_4k_10bit(seed, frame_idx):
    """3840x2160 4:2:2 10-bit frame: range [64, 940], sigma 16, rectangles drifting 2 px per frame."""
    return frame(3840, 2160, 10, FMT_YUV422, seed=seed, frame_idx=frame_idx, lo=64, hi=940, sigma=16, drift=2)
