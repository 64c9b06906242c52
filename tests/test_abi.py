"""C-ABI checks that need no GPU: the library builds for sm_103a, loads,
and exports every function include/vf.h declares; the Python binding
declares the same set; calls fail loudly without a device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "vf.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vf_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    from voxelfragmentml_gb300 import build as B
    return B.build()


def test_header_declares_entry_points():
    names = _declared()
    for must in ("vf_ctx_create", "vf_grid_create", "vf_voxelize", "vf_sample_seeds",
                 "vf_fracture", "vf_fracture_plain", "vf_perturb", "vf_detect_boundaries",
                 "vf_erode", "vf_count_values", "vf_fracture_model", "vf_batch_run",
                 "vf_plain_run", "vf_server_create", "vf_server_submit", "vf_server_poll"):
        assert must in names


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    import voxelfragmentml_gb300 as V
    assert set(_declared()) <= set(V.EXPORTS)


def test_params_default_matches_fracture_parameters(libpath):
    import voxelfragmentml_gb300 as V
    p = V.Params.default()
    # FractureParameters() defaults (FractureParameters.h:91-145)
    assert (p.algorithm, p.distance, p.num_seeds, p.seed) == (V.FLOOD, V.CHEBYSHEV, 8, 80)
    assert (p.erosion_type, p.erosion_size, p.erosion_iterations) == (V.ELLIPSE, 3, 3)
    assert abs(p.erosion_probability - 0.5) < 1e-7 and abs(p.erosion_threshold - 0.5) < 1e-7
    assert p.boundary_size == 1 and p.seed_location == V.OUTER


def test_no_device_fails_loudly(libpath):
    import voxelfragmentml_gb300 as V
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = True
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(V.VFError) as e:
        V.Context(0)
    assert e.value.status == V.ERR_NOT_BUILT


def test_status_strings(libpath):
    import voxelfragmentml_gb300 as V
    L = V.lib()
    assert L.vf_status_string(0) == b"ok"
    assert b"seed" in L.vf_status_string(V.ERR_SEED_SEARCH)
    assert b"sm_103a" in L.vf_version()
