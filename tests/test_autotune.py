"""sparkle_gb300.autotune against a fake context (no GPU): the coordinate descent keeps the fastest setting
per knob, rebuilds the scene only when a BVH knob changes, skips failing settings, and leaves the context
on the best setting it found."""
from sparkle_gb300 import autotune as at

DEFAULTS = dict(cuda_graph=1, material_sort=0, bvh_width=8, bvh_leaf_size=3, extend_blocks_per_sm=0,
                shade_blocks_per_sm=8, batch_slots=0, ray_sort=0, bvh_collapse=0, bvh_builder=0,
                path_slots_per_pixel=64, shadow_stage=1, multi_frame=1, primary_packets=1)


class FakeContext:
    """Device time = a separable cost per knob; the scene knobs only take effect after a rebuild."""

    def __init__(self, cost, fail=None):
        self.knobs = dict(DEFAULTS)
        self.scene = {k: DEFAULTS[k] for k in at.SCENE_KNOBS}
        self.cost = cost
        self.fail = fail or (lambda knobs: False)
        self.rebuilds = 0

    def tuning(self):
        return dict(self.knobs)

    def set_tuning(self, **kw):
        self.knobs.update(kw)

    def rebuild(self):
        self.rebuilds += 1
        self.scene = {k: self.knobs[k] for k in at.SCENE_KNOBS}

    def run(self, _ctx):
        effective = dict(self.knobs, **self.scene)
        ms = 10.0 + sum(self.cost.get(k, {}).get(v, 0.0) for k, v in effective.items())
        return {"extension_rays": 1_000_000, "shadow_rays": 0, "device_ms": ms,
                "error_flags": 1 if self.fail(effective) else 0}


def test_descent_finds_the_separable_optimum():
    cost = {"shade_blocks_per_sm": {16: -1.0}, "bvh_leaf_size": {2: -0.5}, "path_slots_per_pixel": {16: 2.0},
            "material_sort": {1: 3.0}}
    ctx = FakeContext(cost)
    best, hist = at.autotune(ctx, ctx.run, rebuild=ctx.rebuild, log=None)
    assert best["shade_blocks_per_sm"] == 16 and best["bvh_leaf_size"] == 2
    assert best["path_slots_per_pixel"] == 64 and best["material_sort"] == 0
    assert ctx.tuning() == best
    assert ctx.scene["bvh_leaf_size"] == 2  # the final setting's scene was rebuilt
    # one evaluation of the start plus one per non-default value of every knob
    assert len(hist) == 1 + sum(len([v for v in vals if v != DEFAULTS[k]]) for k, vals in at.SPACE.items())


def test_scene_knobs_rebuild_only_when_they_change():
    ctx = FakeContext({})
    at.autotune(ctx, ctx.run, rebuild=ctx.rebuild, log=None)
    scene_values = sum(len([v for v in at.SPACE[k] if v != DEFAULTS[k]]) for k in at.SCENE_KNOBS)
    # each scene-knob candidate rebuilds, and so does the return to the defaults after it
    assert ctx.rebuilds <= 2 * scene_values
    assert ctx.rebuilds >= scene_values


def test_without_rebuild_hook_scene_knobs_are_not_searched():
    ctx = FakeContext({"bvh_width": {4: -5.0}})
    best, hist = at.autotune(ctx, ctx.run, rebuild=None, log=None)
    assert best["bvh_width"] == 8
    assert all(h[0]["bvh_width"] == 8 for h in hist)


def test_failing_settings_are_skipped():
    cost = {"material_sort": {1: -4.0}}
    ctx = FakeContext(cost, fail=lambda knobs: knobs["material_sort"] == 1)
    best, hist = at.autotune(ctx, ctx.run, rebuild=ctx.rebuild, log=None)
    assert best["material_sort"] == 0
    assert any(h[0]["material_sort"] == 1 and h[1] is None for h in hist)
