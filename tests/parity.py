"""Shared comparison helpers of the parity tests (hit records and images), over oracle/compare.py, with the
image tolerances the tests use."""
from __future__ import annotations

from oracle.compare import (INVALID, axis_parallel, classify_hits, close_fraction, compare_images,  # noqa: F401
                            oracle_hits, rel_mse)

# Image parity: the device and the oracle draw the same random numbers and round every multiply and add the
# same way; they differ only in the last bits of cosf/sinf/powf/sqrtf (CUDA's versus the host libm), so a
# path occasionally takes the other branch of a Fresnel, metal or roulette coin and that sample differs. A
# low-spp image is therefore compared per pixel: at least MIN_CLOSE of the pixels within 1e-4 relative, and
# every pixel whose frame-buffer value is bit-identical has a bit-identical tonemapped RGBA16F value. Its
# relMSE is dominated by the few diverged samples (one sample of 16 that reaches the 6.0-clamped light
# instead of a dark wall adds about 1e-4 to a 256x256 image), so it is bounded by MAX_RELMSE_LOW_SPP for
# renders of at most 16 frames and by MAX_RELMSE_CONVERGED for converged renders (256 frames and more),
# where each diverged sample weighs 1/frames.
MIN_CLOSE = 0.995
MAX_RELMSE_LOW_SPP = 1e-3
MAX_RELMSE_CONVERGED = 1e-4


def assert_image_parity(res: dict, label: str = "", min_close: float = MIN_CLOSE,
                        max_relmse: float = MAX_RELMSE_LOW_SPP):
    print(f"{label} pixels={res['pixels']} identical={res['identical']} differing={res['differing']} "
          f"close={res['close']:.5f} relmse={res['relmse']:.3e} tonemap_checked={res.get('tonemap_checked')} "
          f"tonemap_mismatch={res.get('tonemap_mismatch')}")
    assert res["close"] >= min_close, res
    assert res["relmse"] < max_relmse, res
    if "tonemap_mismatch" in res:
        assert res["tonemap_checked"] > 0 and res["tonemap_mismatch"] == 0, res


def oracle_image(scene, camera, cfg, frames, osc=None):
    """The oracle's (frame buffer, RGBA16F image) of `frames` frames of `scene` under `cfg`."""
    import oracle
    osc = osc or oracle.OracleScene(scene)
    r = oracle.OracleRenderer(osc, cfg, camera)
    r.render(frames, traversal=oracle.PRUNED)
    return r.framebuffer()


def assert_hits_match_oracle(got, scene, rays, label: str = "", max_bad_frac: float = 2e-5, osc=None) -> dict:
    """Device closest hits against the oracle's on the same rays: every ray exact, an order-dependent tie at
    bit-identical t, or (rarely) a grazing box test; returns the counts."""
    import oracle
    osc = osc or oracle.OracleScene(scene)
    ref, _ = oracle_hits(osc, rays, oracle.PRUNED)
    c = classify_hits(got, ref)
    print(label, {k: v for k, v in c.items() if k != "mismatch_idx"})
    assert c["other"] == 0
    assert c["gpu_closer"] + c["ref_closer"] <= max(2, max_bad_frac * c["n"])
    assert c["exact"] + c["tie"] >= (1 - max_bad_frac) * c["n"] - 2
    return c
