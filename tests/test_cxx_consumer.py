"""A compiled C++ consumer of the C ABI: tests/cxx/consumer.cpp uses the
header-only facade include/vf.hpp (vf::Grid, vf::Seeder::uniform,
vf::FloodFracturer::build, shaped like RegularGrid, Seeder and
fracturer::Fracturer) over include/vf.h, and links libvfgb300.so.

Without a GPU the program must compile, link, load the library and fail
loudly with VF_ERR_NOT_BUILT; on the GPU its labels, seeds and counts must
equal the oracle's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def consumer(tmp_path_factory):
    from voxelfragmentml_gb300 import build as B
    lib = B.build()
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("cxx") / "consumer")
    libdir = os.path.dirname(lib)
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cxx", "consumer.cpp"), "-o", exe,
           "-L", libdir, "-lvfgb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _grid():
    rng = np.random.default_rng(3)
    occ = (rng.random((26, 21, 37)) < 0.62).astype(np.uint16)
    occ[:, 10, :] = 1  # a connected sheet through the grid
    return occ


def _run(exe, occ, tmp_path, n=6, seed=42, dist=1):
    gpath, opath = str(tmp_path / "grid.bin"), str(tmp_path / "out.bin")
    occ.tofile(gpath)
    X, Y, Z = occ.shape
    r = subprocess.run([exe, gpath, opath, str(X), str(Y), str(Z), str(n), str(seed), str(dist)],
                       capture_output=True, text=True, timeout=300)
    return r, opath


def test_cxx_consumer_links_and_fails_loudly_without_gpu(consumer, tmp_path):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    r, _ = _run(consumer, _grid(), tmp_path)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "device" in r.stderr.lower()


@pytest.mark.gpu
@pytest.mark.parametrize("dist", [1, 2])
def test_cxx_consumer_matches_oracle(consumer, tmp_path, oracle_lib, dist):
    import oracle as O
    occ = _grid()
    r, opath = _run(consumer, occ, tmp_path, dist=dist)
    assert r.returncode == 0, r.stderr
    raw = open(opath, "rb").read()
    ns = int(np.frombuffer(raw[:4], np.uint32)[0])
    off = 4
    seeds = np.frombuffer(raw[off:off + 16 * ns], np.uint32).reshape(ns, 4)
    off += 16 * ns
    labels = np.frombuffer(raw[off:off + 2 * occ.size], np.uint16).reshape(occ.shape)
    off += 2 * occ.size
    counts = np.frombuffer(raw[off:off + 1024], np.uint32)
    occupied = int(np.frombuffer(raw[off + 1024:off + 1032], np.uint64)[0])
    exp_seeds = O.seeder_uniform(occ, 6, 42, 2)
    assert np.array_equal(seeds, exp_seeds)
    lab, _ = O.flood(occ, exp_seeds, dist)
    lab = O.detect_boundaries(lab, 1)
    assert np.array_equal(labels, lab)
    cnt = O.count_values(lab, 256)
    cnt = cnt[0] if isinstance(cnt, tuple) else cnt
    assert np.array_equal(counts, cnt)
    assert occupied == int(cnt.sum())
