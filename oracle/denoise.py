"""Test infrastructure only (the checker, never shipped or measured): a NumPy restatement of
the `denoise` post-processor's edge-avoiding a-trous wavelet filter.

The reference's `denoise` post-processor (src/builtin/btrc/builtin/postprocess/
optix_denoiser.cpp:51-126) runs the OptiX AI denoiser, a closed library; the product
replaces it with the published filter of Dammertz, Sewtz, Hanika and Lensch, "Edge-Avoiding
A-Trous Wavelet Transform for fast Global Illumination Filtering" (HPG 2010). There is no
reference output to pin this against (parity unpinned): this restatement checks the CUDA
kernel against the method's definition.

Pass k (k = 0..4) convolves with the 5x5 B3-spline kernel (1/16, 1/4, 3/8, 1/4, 1/16)
dilated to a tap spacing of 2^k; tap q of pixel p is weighted by
exp(-(|T(c_p) - T(c_q)|^2 / sigma_c,k^2 + |a_p - a_q|^2 / sigma_a^2 + |n_p - n_q|^2 / (4^k sigma_n^2)))
with T(c) = max(c, 0) / (1 + max(c, 0)) per channel and sigma_c,k = sigma_c / 2^k; the albedo and
normal terms drop out when that guide is absent; taps outside the image are skipped and
the weights renormalised. FP32 throughout, taps accumulated row by row as the kernel does.
"""
import numpy as np

PASSES = 5
SIGMA_COLOR = 0.5
SIGMA_ALBEDO = 0.05
SIGMA_NORMAL = 0.3
_H = np.array([0.375, 0.25, 0.0625], np.float32)


def _tone(c: np.ndarray) -> np.ndarray:
    c = np.maximum(c, np.float32(0))
    return (c / (np.float32(1) + c)).astype(np.float32)


def atrous_pass(img: np.ndarray, albedo: np.ndarray | None, normal: np.ndarray | None, step: int,
                inv_sc2: np.float32, inv_sa2: np.float32, inv_sn2: np.float32) -> np.ndarray:
    h, w, _ = img.shape
    f32 = np.float32
    tp = _tone(img)
    sums = np.zeros((h, w, 3), f32)
    sw = np.zeros((h, w), f32)
    ys, xs = np.arange(h), np.arange(w)
    for dy in range(-2, 3):
        qy = ys + dy * step
        vy = (qy >= 0) & (qy < h)
        qyc = np.clip(qy, 0, h - 1)
        for dx in range(-2, 3):
            qx = xs + dx * step
            vx = (qx >= 0) & (qx < w)
            qxc = np.clip(qx, 0, w - 1)
            valid = vy[:, None] & vx[None, :]
            cq = img[qyc][:, qxc]
            d = tp - _tone(cq)
            e = (d * d).sum(-1, dtype=f32) * inv_sc2
            if albedo is not None:
                d = albedo - albedo[qyc][:, qxc]
                e = (e + (d * d).sum(-1, dtype=f32) * inv_sa2).astype(f32)
            if normal is not None:
                d = normal - normal[qyc][:, qxc]
                e = (e + (d * d).sum(-1, dtype=f32) * inv_sn2).astype(f32)
            wt = (_H[abs(dx)] * _H[abs(dy)] * np.exp(-e).astype(f32)).astype(f32)
            wt = np.where(valid, wt, f32(0))
            sums += wt[..., None] * cq
            sw += wt
    return (sums / sw[..., None]).astype(f32)


def atrous(img: np.ndarray, albedo: np.ndarray | None = None, normal: np.ndarray | None = None) -> np.ndarray:
    """(H, W, 3) float32 image (and optional (H, W, 3) guides) -> denoised (H, W, 3) float32."""
    f32 = np.float32
    out = np.ascontiguousarray(img, f32)
    alb = None if albedo is None else np.ascontiguousarray(albedo, f32)
    nrm = None if normal is None else np.ascontiguousarray(normal, f32)
    for k in range(PASSES):
        step = f32(1 << k)
        sc = f32(SIGMA_COLOR) / step
        out = atrous_pass(out, alb, nrm, 1 << k, f32(1) / (sc * sc), f32(1) / (f32(SIGMA_ALBEDO) * f32(SIGMA_ALBEDO)),
                          f32(1) / (f32(SIGMA_NORMAL) * f32(SIGMA_NORMAL) * step * step))
    return out
