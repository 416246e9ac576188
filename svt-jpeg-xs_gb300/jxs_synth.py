"""Seeded synthetic frames for the JPEG XS encode/decode workloads.

Content model for one plane: a smooth 2-D linear gradient, approximately
Gaussian noise, and axis-aligned rectangles with uniform random fill (hard
edges), clipped to the sample range.  8-bit planes use the gradient range
[16, 235] and noise sigma 4; other depths rescale that model by
(2^d - 1) / 255 unless a range and sigma are given (the 4K 10-bit stream uses
[64, 940] and sigma 16).  Rectangles may drift by `drift` pixels per frame.

Everything is integer arithmetic on numpy's PCG64 integer stream, so a seed
gives bit-identical frames on every platform: noise is the sum of four
uniform integers in [-r, r] (variance 4 r (r + 1) / 3, r chosen for the
requested sigma), drawn as int16.
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


def _noise_radius(sigma):
    r = 0
    while 4 * (r + 1) * (r + 2) / 3.0 <= sigma * sigma:
        r += 1
    return r


def plane(rng, w, h, depth, frame_idx=0, lo=None, hi=None, sigma=None, rects=20, drift=0, noise_quadrant=False):
    maxv = (1 << depth) - 1
    if lo is None:
        lo = (16 * maxv) // 255
    if hi is None:
        hi = (235 * maxv) // 255
    if sigma is None:
        sigma = 4.0 * maxv / 255.0
    x = np.arange(w, dtype=np.int64)[None, :]
    y = np.arange(h, dtype=np.int64)[:, None]
    dx, dy = max(w - 1, 1), max(h - 1, 1)
    img = lo + ((hi - lo) * (x * dy + y * dx)) // (2 * dx * dy)
    r = _noise_radius(sigma)
    if r:
        img = img + rng.integers(-r, r + 1, size=(4, h, w), dtype=np.int16).sum(axis=0, dtype=np.int64)
    for _ in range(rects):
        x0, x1 = np.sort(rng.integers(0, w, size=2))
        y0, y1 = np.sort(rng.integers(0, h, size=2))
        val = int(rng.integers(0, maxv + 1))
        d = drift * frame_idx
        xa, xb = min(w, x0 + d), min(w, x1 + 1 + d)
        img[y0:y1 + 1, xa:xb] = val
    if noise_quadrant:
        img[: h // 2, : w // 2] = rng.integers(0, maxv + 1, size=(h // 2, w // 2))
    img = np.clip(img, 0, maxv)
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


def frame_8k_14bit(seed, frame_idx=0):
    """7680x4320 planar RGB (gbrp) 14-bit: uniform 14-bit noise in one quarter, gradient + rectangles elsewhere."""
    return frame(7680, 4320, 14, FMT_YUV444, seed=seed, frame_idx=frame_idx, noise_quadrant=True)
