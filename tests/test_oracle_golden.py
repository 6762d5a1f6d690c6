"""The oracle (C restatement of the reference pipeline) against golden
fixtures rendered by the reference's own pipeline core, and -- where the
reference sources are present -- against that build directly."""
import numpy as np
import pytest

from common import assert_depth_exact, load_golden, render, sha
from cpu_backends import OraclePipeline, RefPipeline, ref_available
from golden.make_golden import golden_cases, scene_digest

CASES = golden_cases()


@pytest.mark.parametrize("name,scene", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_golden(name, scene):
    g = load_golden(name)
    if scene_digest(scene) != str(g["digest"]):
        pytest.skip("scene inputs generated on this host differ from the fixture's (float library differences)")
    out = render(OraclePipeline(scene.width, scene.height), scene)
    if "depth" in g:
        assert_depth_exact(out["depth"], g["depth"], name)
        assert np.array_equal(out["colour"], g["colour"]), name
    assert sha(out["depth"]) == str(g["depth_sha"]), name
    assert sha(out["colour"]) == str(g["colour_sha"]), name
    if "shadow_sha" in g:
        assert sha(out["shadow"]) == str(g["shadow_sha"]), name
    assert int((out["depth"] < 1.0).sum()) == int(g["covered"])


@pytest.mark.skipif(not ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("threads", [1, 3])
def test_oracle_thread_count_invariant(threads):
    """Row partitioning across threads never changes the result (per-row FIFO order)."""
    name, scene = CASES[4]
    a = render(OraclePipeline(scene.width, scene.height, threads=threads), scene)
    b = render(RefPipeline(scene.width, scene.height), scene)
    assert_depth_exact(a["depth"], b["depth"], name)
    assert np.array_equal(a["colour"], b["colour"])
