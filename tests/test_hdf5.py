"""HDF5 ingest and export of the CLI (host/hdf5.cpp, reached through
``knng_main --h5dump`` / ``--convert``) and the numpy reader hdf5read.py.

The reference reads /train with libhdf5 and writes knns/dists plus the
attributes algo, task, buildtime, querytime, params (src/main.cpp:101-112,
149-177, 464-480).  Both readers are checked against the one libhdf5-written
file on the image (scipy's MATLAB v7.3 test file, when scipy ships it),
against generated fixtures of the other layouts libhdf5 writes
(tests/golden/hdf5/make_hdf5.py), and the writer through both readers."""
import glob
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sisap-2026-task1_gb300")
GOLD = os.path.join(ROOT, "tests", "golden", "hdf5")
CLI = os.path.join(PKG, "knng_main")


@pytest.fixture(scope="module")
def cli():
    import importlib.util

    spec = importlib.util.spec_from_file_location("knng_build_script", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    return CLI


def h5dump(cli, path, name=None):
    r = subprocess.run([cli, "--h5dump", str(path)] + ([name] if name else []), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout, parse_int=float if name else int)  # values: keep "-0" as -0.0


def libhdf5_file():
    try:
        import scipy.io
    except ImportError:
        return None
    hits = glob.glob(os.path.join(os.path.dirname(scipy.io.__file__), "matlab", "tests", "data", "testhdf5_7.4_GLNX86.mat"))
    return hits[0] if hits else None


def test_libhdf5_written_file_both_readers(cli):
    path = libhdf5_file()
    if path is None:
        pytest.skip("scipy's libhdf5-written MATLAB v7.3 test file is not installed")
    import hdf5read

    want = np.arange(9, dtype=np.float64) * (np.pi / 4)  # MATLAB testdouble = 0:pi/4:2*pi
    ds, _ = hdf5read.read(path)
    assert list(ds) == ["testdouble"] and ds["testdouble"].dtype == np.float64 and ds["testdouble"].shape == (9, 1)
    np.testing.assert_allclose(ds["testdouble"].ravel(), want, rtol=0, atol=1e-15)
    assert hdf5read.attributes(path, "testdouble") == {"MATLAB_class": "double"}
    out = h5dump(cli, path, "testdouble")
    assert out["datasets"] == [{"name": "testdouble", "class": 1, "size": 8, "little_endian": True, "signed": True,
                                "dims": [9, 1]}]
    assert np.array_equal(np.float32(out["values"]), want.astype(np.float32))


def expected():
    z = np.load(os.path.join(GOLD, "h5_expected.npz"))
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("fixture,prefix", [("h5_v0_chunked.h5", "v0"), ("h5_v2_links.h5", "v2")])
def test_cpp_reader_generated_fixtures(cli, fixture, prefix):
    path = os.path.join(GOLD, fixture)
    exp = {k.split(":", 1)[1]: v for k, v in expected().items() if k.startswith(prefix + ":")}
    out = h5dump(cli, path)
    listed = {d["name"]: d for d in out["datasets"]}
    assert sorted(listed) == sorted(exp)
    for name, want in exp.items():
        d = listed[name]
        assert d["dims"] == list(want.shape)
        assert d["size"] == want.dtype.itemsize and d["class"] == (1 if want.dtype.kind == "f" else 0)
        assert d["little_endian"] == (name != "ids")  # the fixture stores "ids" big-endian
        got = np.float32(h5dump(cli, path, name)["values"]).reshape(want.shape)
        assert np.array_equal(got, want.astype(np.float32)), name
    if prefix == "v0":
        assert out["attrs"] == {"title": "knng fixture", "note": "variable length value"}
        assert np.signbit(np.float32(h5dump(cli, path, "train")["values"])[3 * 10 + 7])  # -0.0 kept
    else:
        assert out["attrs"] == {"version": "2.5"}


@pytest.mark.parametrize("fixture,prefix", [("h5_v0_chunked.h5", "v0"), ("h5_v2_links.h5", "v2")])
def test_python_reader_generated_fixtures(fixture, prefix):
    import hdf5read

    ds, attrs = hdf5read.read(os.path.join(GOLD, fixture))
    exp = {k.split(":", 1)[1]: v for k, v in expected().items() if k.startswith(prefix + ":")}
    # Version 4 chunk indexes (single / implicit / fixed array) are the C++ reader's alone.
    skip = {"single", "implicit", "fixed"} if prefix == "v2" else set()
    assert sorted(ds) == sorted(set(exp) - skip)
    for name in ds:
        assert ds[name].dtype.str[1:] == exp[name].dtype.str[1:], name
        assert ds[name].dtype.byteorder == (">" if name == "ids" else exp[name].dtype.byteorder)
        assert np.array_equal(ds[name], exp[name]), name
    assert attrs == ({"title": "knng fixture", "note": "variable length value"} if prefix == "v0" else {"version": 2.5})


def result_arrays(rows=33, k=15, seed=3):
    rng = np.random.default_rng(seed)
    knns = rng.integers(1, 1 << 31, size=(rows, k)).astype(np.int32)
    dists = rng.standard_normal((rows, k)).astype(np.float32)
    dists[0, 0] = -0.0
    return knns, dists


def test_writer_through_both_readers(cli, tmp_path):
    import h5container
    import hdf5read

    knns, dists = result_arrays()
    params = "K_BUILD=50, RERANK=8, TREES=16, LEAF=64, STOP=0.04, DIFF=0.01"
    h5container.write(tmp_path / "r.knng", {"knns": knns, "dists": dists},
                      {"algo": "knng \"GB300\"\\x", "task": "task1", "params": params},
                      {"buildtime": 4.25, "querytime": 0.0})
    assert subprocess.run([cli, "--convert", str(tmp_path / "r.knng"), str(tmp_path / "r.h5")]).returncode == 0
    raw = open(tmp_path / "r.h5", "rb").read()
    assert raw[:8] == b"\x89HDF\r\n\x1a\n" and raw[8] == 0  # superblock version 0, as libhdf5's default
    assert int.from_bytes(raw[40:48], "little") == len(raw)  # end-of-file address
    ds, at = hdf5read.read(tmp_path / "r.h5")
    assert sorted(ds) == ["dists", "knns"]
    assert ds["knns"].dtype == np.int32 and np.array_equal(ds["knns"], knns)
    assert ds["dists"].dtype == np.float32 and np.array_equal(ds["dists"].view(np.uint32), dists.view(np.uint32))
    assert at == {"algo": "knng \"GB300\"\\x", "task": "task1", "buildtime": 4.25, "querytime": 0.0, "params": params}
    out = h5dump(cli, tmp_path / "r.h5", "knns")
    assert np.array_equal(np.float32(out["values"]).reshape(knns.shape), knns.astype(np.float32))  # dumped as f32
    assert out["attrs"]["params"] == params and out["attrs"]["buildtime"] == "4.25"
    # Back to a container: bit-identical arrays and attributes.
    assert subprocess.run([cli, "--convert", str(tmp_path / "r.h5"), str(tmp_path / "r2.knng"),
                           "--output-format", "knng"]).returncode == 0
    ds2, at2 = h5container.read(tmp_path / "r2.knng", mmap=False)
    assert np.array_equal(ds2["knns"], knns) and np.array_equal(ds2["dists"].view(np.uint32), dists.view(np.uint32))
    assert at2 == at


def test_writer_empty_result(cli, tmp_path):
    import h5container
    import hdf5read

    h5container.write(tmp_path / "e.knng", {"knns": np.zeros((0, 15), np.int32), "dists": np.zeros((0, 15), np.float32)},
                      {"algo": "", "task": "t", "params": ""}, {"buildtime": 0.0, "querytime": 0.0})
    assert subprocess.run([cli, "--convert", str(tmp_path / "e.knng"), str(tmp_path / "e.h5")]).returncode == 0
    ds, at = hdf5read.read(tmp_path / "e.h5")
    assert ds["knns"].shape == (0, 15) and ds["dists"].shape == (0, 15)
    assert at["algo"] == "" and at["task"] == "t"


def test_cli_reads_hdf5_train_and_rejects_bad_files(cli, tmp_path):
    # /train of a chunked, deflated HDF5 file is found and read (the build that
    # follows needs a GPU: without one the CLI stops with the reference's -1).
    r = subprocess.run([cli, os.path.join(GOLD, "h5_v0_chunked.h5")], capture_output=True, text=True, cwd=tmp_path)
    assert "[OK] Detected 40 vectors in /train." in r.stdout and r.returncode in (0, 255), r.stderr
    # A result file has no /train.
    knns, dists = result_arrays()
    import h5container

    h5container.write(tmp_path / "r.knng", {"knns": knns, "dists": dists}, {}, {})
    assert subprocess.run([cli, "--convert", str(tmp_path / "r.knng"), str(tmp_path / "r.h5")]).returncode == 0
    r = subprocess.run([cli, "r.h5"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 255 and "Dataset Error" in r.stderr and "/train" in r.stderr
    (tmp_path / "junk.h5").write_bytes(b"not an hdf5 file at all" * 40)
    r = subprocess.run([cli, "--h5dump", str(tmp_path / "junk.h5")], capture_output=True, text=True)
    assert r.returncode == 255 and "superblock" in r.stderr
    good = open(os.path.join(GOLD, "h5_v0_chunked.h5"), "rb").read()
    (tmp_path / "cut.h5").write_bytes(good[:2000])
    r = subprocess.run([cli, "--h5dump", str(tmp_path / "cut.h5"), "train"], capture_output=True, text=True)
    assert r.returncode == 255 and "HDF5" in r.stderr


def test_user_block_offset(cli, tmp_path):
    """A file with a 512-byte user block (as MATLAB writes) keeps its addresses
    relative to the superblock."""
    import hdf5read

    good = open(os.path.join(GOLD, "h5_v0_chunked.h5"), "rb").read()
    (tmp_path / "ub.h5").write_bytes(b"U" * 512 + good)
    ds, _ = hdf5read.read(tmp_path / "ub.h5")
    exp = expected()["v0:train"]
    assert np.array_equal(ds["train"], exp)
    got = np.float32(h5dump(cli, tmp_path / "ub.h5", "train")["values"]).reshape(exp.shape)
    assert np.array_equal(got, exp)


WRITER_DRIVER = r"""
#include "hdf5.h"
#include <cstdint>
#include <vector>
int main(int, char** argv) {
  std::vector<uint16_t> half(6 * 4);
  for (int i = 0; i < 24; ++i) half[i] = uint16_t(0x3c00 + i);  // 1.0, 1.0009765625, ...
  std::vector<int32_t> knns(6 * 3);
  std::vector<float> dists(6 * 3);
  for (int i = 0; i < 18; ++i) { knns[i] = 7 * i + 1; dists[i] = 0.25f * float(i) - 2.0f; }
  knngio::h5::write_file(argv[1], {{"train", 2, {6, 4}, half.data()},
                                   {"allknn/knns", 0, {6, 3}, knns.data()},
                                   {"allknn/dists", 1, {6, 3}, dists.data()}},
                         {{"note", true, "groups and halves", 0.0f}});
  return 0;
}
"""


def test_writer_groups_and_f16(cli, tmp_path):
    """The writer's float16 datasets and one group level, read back by both readers."""
    import hdf5read

    src = tmp_path / "drv.cpp"
    src.write_text(WRITER_DRIVER)
    exe = tmp_path / "drv"
    subprocess.run(["g++", "-std=c++20", "-O1", "-I", os.path.join(PKG, "host"), str(src),
                    os.path.join(PKG, "host", "hdf5.cpp"), "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(tmp_path / "g.h5")], check=True)
    ds, at = hdf5read.read(tmp_path / "g.h5")
    assert sorted(ds) == ["allknn/dists", "allknn/knns", "train"]
    want_half = (np.arange(24, dtype=np.uint16) + 0x3C00).view(np.float16).reshape(6, 4)
    assert ds["train"].dtype == np.float16 and np.array_equal(ds["train"], want_half)
    assert np.array_equal(ds["allknn/knns"], (7 * np.arange(18) + 1).reshape(6, 3).astype(np.int32))
    assert np.array_equal(ds["allknn/dists"], (0.25 * np.arange(18) - 2).reshape(6, 3).astype(np.float32))
    assert at == {"note": "groups and halves"}
    out = h5dump(cli, tmp_path / "g.h5", "train")
    assert {d["name"] for d in out["datasets"]} == {"train", "allknn/knns", "allknn/dists"}
    assert np.array_equal(np.float32(out["values"]).reshape(6, 4), want_half.astype(np.float32))


@pytest.mark.parametrize("fixture", ["h5_v0_chunked.h5", "h5_v2_links.h5"])
def test_reader_survives_corrupt_files(cli, tmp_path, fixture):
    """Random byte changes and truncations of a valid file make the reader
    either succeed or fail with its -1 status and a message, never crash."""
    import random

    good = open(os.path.join(GOLD, fixture), "rb").read()
    rng = random.Random(len(good))
    path = tmp_path / "bad.h5"
    for trial in range(40):
        data = bytearray(good)
        if trial % 5 == 4:
            data = data[: rng.randrange(8, len(data))]
        else:
            for _ in range(rng.randrange(1, 9)):
                data[rng.randrange(len(data))] = rng.randrange(256)
        path.write_bytes(bytes(data))
        for name in (None, "train"):
            r = subprocess.run([cli, "--h5dump", str(path)] + ([name] if name else []), capture_output=True,
                               text=True, timeout=30)
            assert r.returncode in (0, 255), (trial, r.returncode, r.stderr[-200:])


def test_cli_reads_float16_train(cli, tmp_path):
    """A float16 /train (what the reference's PCA script writes) is read and
    widened to float32 by the CLI (the build that follows needs a GPU)."""
    import sys

    sys.path.insert(0, GOLD)
    import make_hdf5

    x = np.random.default_rng(9).standard_normal((300, 128)).astype(np.float16)
    make_hdf5.write_datasets(tmp_path / "h.h5", {"train": x}, chunks=(64, 128), deflate=True)
    out = h5dump(cli, tmp_path / "h.h5", "train")
    assert out["datasets"][0]["size"] == 2 and out["datasets"][0]["class"] == 1
    assert np.array_equal(np.float32(out["values"]).reshape(300, 128), x.astype(np.float32))
    r = subprocess.run([cli, "h.h5"], capture_output=True, text=True, cwd=tmp_path)
    assert "[OK] Detected 300 vectors in /train." in r.stdout and r.returncode in (0, 255), r.stderr
