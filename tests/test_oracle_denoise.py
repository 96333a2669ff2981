"""Properties of the denoise filter's restatement (oracle/denoise.py) that the method
defines: normalised weights, edge stopping on the guides, noise reduction."""
import numpy as np

from oracle import denoise as OD


def test_constant_image_is_unchanged():
    img = np.full((33, 47, 3), [0.2, 1.5, 7.0], np.float32)
    out = OD.atrous(img)
    assert np.allclose(out, img, rtol=1e-6)


def test_albedo_edge_is_not_blurred():
    # two regions of different albedo, each a constant colour: the albedo term stops the
    # filter at the boundary, so each side keeps its own colour
    h, w = 32, 64
    alb = np.zeros((h, w, 3), np.float32)
    alb[:, : w // 2] = 0.2
    alb[:, w // 2:] = 0.8
    img = np.where(np.arange(w)[None, :, None] < w // 2, 0.1, 5.0).astype(np.float32) * np.ones((h, w, 3), np.float32)
    out = OD.atrous(img, albedo=alb)
    assert np.allclose(out[:, : w // 2], 0.1, rtol=1e-4)
    assert np.allclose(out[:, w // 2:], 5.0, rtol=1e-4)
    # without the guide the colour term alone still separates colours this far apart
    # except right at the edge, where the filter mixes them a little
    plain = OD.atrous(img)
    assert np.abs(plain - img).max() > np.abs(out - img).max()


def test_noise_is_reduced_in_flat_regions():
    rng = np.random.default_rng(5)
    img = (0.5 * rng.exponential(1.0, (64, 64, 3))).astype(np.float32)
    out = OD.atrous(img, albedo=np.full_like(img, 0.5), normal=np.broadcast_to(np.float32([0, 0, 1]), img.shape))
    assert out.std() < 0.3 * img.std()
    assert abs(out.mean() - img.mean()) < 0.1 * img.mean()
