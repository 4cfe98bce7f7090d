"""The CUDA pipeline, through the C ABI, against the reference's own compute
shaders: for every scene of tests/golden/reference_shaders.npz (frames of the
reference's Slang source run on the CPU; see tests/test_reference_shaders.py)
the key count, the splats, the sorted keys and values and the tile ranges
are bit-exact, and the image agrees within 1e-3 per channel with the
reference's (the fixture's, or for large images the oracle's FP32
transcription, whose digest equals the reference's) outside the pixels whose
FP64 decisions lie at a threshold."""
import numpy as np
import pytest

import torpedo_gb300 as T
from oracle import oracle as O
from tests.golden import shader_scenes as SS
from tests.tolerances import IMAGE_ABS
from torpedo_gb300 import _lib as L

pytestmark = pytest.mark.gpu

# scenes of long, thin, rotated Gaussians (condition numbers near 3e4)
ILL_CONDITIONED = {"thin_rotated"}


@pytest.fixture(scope="module")
def fixture():
    return SS.load_fixture()


def _render(d):
    cam = T.Camera(d["view"], d["proj"], d["width"], d["height"])
    np.testing.assert_array_equal(cam.projview().view(np.uint32), d["projview"].view(np.uint32))
    eng = T.GaussianEngine(sh_degree=d["sh_degree"])
    if "ent_idx" in d:
        tr = d["transforms"].reshape(-1, 4, 4)
        eng.compile(d["records"], d["ent_idx"], tr.shape[0])
        for e, m in enumerate(tr):
            eng.transform_host.transform(e, m)
    else:
        eng.compile(d["records"])
    eng.set_camera(cam)
    st = eng.raster_frame()
    n, k = d["n"], st["keys"]
    out = dict(K=k,
               splats=eng.read_buffer(L.TPD_BUF_SPLATS, np.uint32, n * 12).reshape(n, 12),
               keys=eng.read_buffer(L.TPD_BUF_KEYS, np.uint64, k),
               vals=eng.read_buffer(L.TPD_BUF_VALUES, np.uint32, k),
               ranges=eng.read_buffer(L.TPD_BUF_RANGES, np.uint32, st["tiles"] * 2).reshape(-1, 2),
               image=eng.read_image()[0])
    eng.close()
    return out


@pytest.mark.parametrize("name", sorted(SS.build_scenes()))
def test_pipeline_equals_reference_shaders(cuda, fixture, name):
    d = fixture[name]
    g = _render(d)
    assert g["K"] == d["K"], (g["K"], d["K"])
    for k in ("splats", "keys", "vals", "ranges"):
        assert SS.digest(g[k]) == str(d[f"sha_{k}"]), f"{name}: {k} differs from the reference shaders"
    oc = O.camera(d["view"], d["projview"], d["width"], d["height"], focal=tuple(float(x) for x in d["focal"]))
    if name in ILL_CONDITIONED:
        # FP32 conics of these carry up to 2e-3 relative error, in the
        # reference's arithmetic as in ours: the image is held to an FP64 blend
        # of the exact FP32 splats (whose bits the reference's equal), as
        # tests/test_gpu_pipeline.py::test_thin_rotated_needles does
        s64 = g["splats"].view(np.float32).astype(np.float64)
        s64[:, 3] = g["splats"][:, 3].astype(np.float64)
        img64, _, _, pfrag = O.blend_f64(s64, g["vals"], g["ranges"], d["width"], d["height"])
        err = np.abs(g["image"].astype(np.float64) - img64).max(axis=2)[~pfrag]
        assert (err > IMAGE_ABS).sum() <= err.size // 1000, f"{name}: {(err > IMAGE_ABS).sum()} pixels above 1e-3"
        return
    if "image" in d:
        ref = d["image"]
    else:
        # the oracle's FP32 transcription, equal bit for bit to the reference
        # shaders' image (tests/test_reference_shaders.py checks its digest)
        s32 = O.preprocess_f32(d["records"], oc, d["sh_degree"], True, d.get("ent_idx"), d.get("transforms"))
        ref = O.blend_f32(s32, g["vals"], g["ranges"], d["width"], d["height"])[0]
    s64, _, _ = O.preprocess_f64(d["records"], oc, d["sh_degree"], True, d.get("ent_idx"), d.get("transforms"))
    *_, pfrag = O.blend_f64(s64, g["vals"], g["ranges"], d["width"], d["height"])
    err = np.abs(g["image"].astype(np.float64) - ref).max(axis=2)[~pfrag]
    assert err.size == 0 or err.max() <= IMAGE_ABS, f"{name}: image error {err.max()}"
