"""GPU against the reference's own outputs (golden fixtures produced by the
unmodified reference): kNN neighbours and distances, box and radius hit sets,
return values of every mutation and the final set of valid points."""
import pytest

import golden_check as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("replay", G.REPLAYS_TREE, ids=lambda f: f.__name__)
def test_gpu_reproduces_reference_fixtures(ikdg_mod, replay):
    replay(lambda d, b, box: G.Adapter(ikdg_mod.KDTree(d, b, box), "gpu"))
