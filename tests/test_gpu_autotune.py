"""Every launch shape the autotuner can choose gives the oracle's results;
the tuner returns valid choices; the automatic kNN choice equals both kernels."""
import numpy as np
import pytest

from tests.gpu_util import assert_kps_equal, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = require_gpu()
    yield t
    from orb_slam2_detailed_comments_gb300 import autotune
    autotune.apply({"resize_rows": 36, "fast_cells_per_block": 4, "describe_group": 1, "describe_depth": 2, "knn_tc_min_pairs": 1 << 28})
    autotune.apply(autotune.POLICIES)


def frames():
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    return [(syn.scene(1280, 720, 301), 2000), (syn.scene(640, 480, 302), 1000), (syn.scene(1241, 376, 303), 1500)]


@pytest.fixture(scope="module")
def refs(oracle):
    return [oracle.extract(img, nfeatures=nf, want_pyramid=False) for img, nf in frames()]


# every tuned shape under the full-size policies (the three-frame batch would
# otherwise take the small-launch shapes), then every policy value: fixed
# descriptor task sizes and FAST chunks, 8-row or tuned strips for a short
# launch, and the automatic choices
SHAPES = [("resize_rows", 8), ("resize_rows", 22), ("resize_rows", 64), ("fast_cells_per_block", 1),
          ("fast_cells_per_block", 2), ("fast_cells_per_block", 4), ("describe_group", 1), ("describe_group", 2),
          ("describe_group", 4), ("describe_depth", 2), ("describe_depth", 4), ("describe_task", 8),
          ("describe_task", 16), ("describe_task", 32), ("describe_task", 0), ("fast_chunk", 1), ("fast_chunk", 2),
          ("fast_chunk", 4), ("fast_chunk", 0), ("strip_rows_small", 8), ("strip_rows_small", 0)]


@pytest.mark.parametrize("name,value", SHAPES)
def test_batch_shapes_match_oracle(torch, refs, name, value):
    from orb_slam2_detailed_comments_gb300 import autotune
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    defaults = autotune.current()
    try:
        autotune.apply(autotune.FULL_SIZE)
        if name == "strip_rows_small":
            autotune.set_param("resize_rows", 22)
        autotune.set_param(name, value)
        fr = frames()
        b = BatchExtractor(4, 1280, 720, 2000)
        cap = b.per_frame_capacity
        imgs = [torch.from_numpy(img).cuda() for img, _ in fr]
        for _ in range(2):  # plain launch, then the replayed graph
            k, d, c = b.extract(imgs, [nf for _, nf in fr])
        k = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
        d = d.cpu().numpy().reshape(len(fr), cap, 32)
        c = c.cpu().numpy()
        for f, ref in enumerate(refs):
            assert c[f] == len(ref.keypoints)
            assert_kps_equal(k[f, :c[f]], ref.keypoints, f"{name}={value} frame {f}")
            assert np.array_equal(d[f, :c[f]], ref.descriptors)
    finally:
        autotune.apply({k_: v for k_, v in defaults.items() if k_ != "knn_tc_min_pairs"})


def test_per_frame_extractor_replans_after_a_change(torch, refs):
    from orb_slam2_detailed_comments_gb300 import ORBextractor, autotune
    img, nf = frames()[0]
    ex = ORBextractor(nf, 1.2, 8, 20, 7)
    ex(img)
    defaults = autotune.current()
    try:
        autotune.apply({"resize_rows": 8, "fast_cells_per_block": 2, "describe_group": 1})
        k, d = ex(img)
        assert_kps_equal(k, refs[0].keypoints, "replanned")
        assert np.array_equal(d, refs[0].descriptors)
    finally:
        autotune.apply({k_: v for k_, v in defaults.items() if k_ != "knn_tc_min_pairs"})


def test_tuner_choices_and_knn_auto(torch):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher, autotune
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    fr = frames()
    b = BatchExtractor(4, 1280, 720, 2000)
    imgs = [torch.from_numpy(img).cuda() for img, _ in fr]
    policies = {name: autotune.get_param(name) for name in autotune.POLICIES}
    entry = autotune.tune_batch(b, imgs, [nf for _, nf in fr], reps=2)
    for name, (values, _) in autotune.PARAMS.items():
        assert entry[name]["value"] in values
        assert autotune.get_param(name) == entry[name]["value"]
    # the small-launch policies are back as they were
    assert {name: autotune.get_param(name) for name in autotune.POLICIES} == policies
    m = ORBmatcher()
    kn = autotune.tune_knn(m, sizes=((1000, 4000), (4000, 16000)))
    assert kn["value"] > 0 and autotune.get_param("knn_tc_min_pairs") == kn["value"]
    q = torch.from_numpy(syn.random_descriptors(3000, 9)).cuda()
    t = torch.from_numpy(syn.random_descriptors(10000, 10)).cuda()
    ref = m.knn2(q, t, algo=0)
    for threshold in (0, 1 << 62):  # forces each kernel through the automatic choice
        autotune.set_param("knn_tc_min_pairs", threshold)
        out = m.knn2(q, t, algo=-1)
        for a, b_ in zip(out, ref):
            assert torch.equal(a, b_)
