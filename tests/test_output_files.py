"""RSF writers of the output path against the reference's own
original/utils.c (compiled into oracle/_ref by `make -C oracle ref`): the
same calls must produce byte-identical header and binary files.  Host code
only; no GPU needed."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT, reference_dir

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libfletcher_ref.so")
FP = C.POINTER(C.c_float)


@pytest.fixture(scope="module")
def ref():
    if reference_dir() is None:
        pytest.skip("reference sources absent (FLETCHER_REF_DIR or staged copy)")
    import subprocess

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True, capture_output=True)
    lib = C.CDLL(REF_LIB)
    lib.DumpFieldToFile.argtypes = [C.c_int] * 9 + [C.c_float] * 3 + [FP, C.c_char_p]
    lib.OpenSliceFile.restype = C.c_void_p
    lib.OpenSliceFile.argtypes = [C.c_int] * 6 + [C.c_float] * 4 + [C.c_char_p]
    lib.DumpSliceFile.argtypes = [C.c_int] * 3 + [FP, C.c_void_p]
    lib.CloseSliceFile.argtypes = [C.c_void_p]
    return lib


def files(d, name):
    with open(os.path.join(d, name + ".rsf"), "rb") as f:
        head = f.read()
    with open(os.path.join(d, name + ".rsf@"), "rb") as f:
        data = f.read()
    return head, data


def fptr(a):
    return a.ctypes.data_as(FP)


def test_dump_field_to_file_matches_reference(ref, lib, tmp_path, monkeypatch):
    sx, sy, sz = 13, 9, 7
    a = np.random.default_rng(0).standard_normal(sx * sy * sz).astype(np.float32)
    monkeypatch.chdir(tmp_path)
    box = (2, 10, 1, 7, 0, 5)
    ref.DumpFieldToFile(sx, sy, sz, *box, 12.5, 12.5, 10.0, fptr(a), b"r_field")
    assert lib.FLETCHER_DumpFieldToFile(sx, sy, sz, *box, 12.5, 12.5, 10.0, fptr(a), b"g_field") == 0
    rh, rd = files(tmp_path, "r_field")
    gh, gd = files(tmp_path, "g_field")
    assert gh == rh.replace(b"r_field", b"g_field")
    assert gd == rd


@pytest.mark.parametrize("box", [(4, 4, 1, 7, 0, 5), (2, 10, 3, 3, 0, 5), (2, 10, 1, 7, 2, 2), (2, 10, 1, 7, 0, 5)])
def test_slice_files_match_reference(ref, lib, tmp_path, monkeypatch, box):
    """x-, y-, z-slices and a full section, three frames each."""
    sx, sy, sz = 13, 9, 7
    g = np.random.default_rng(1)
    frames = [g.standard_normal(sx * sy * sz).astype(np.float32) for _ in range(3)]
    monkeypatch.chdir(tmp_path)
    rs = ref.OpenSliceFile(*box, 12.5, 12.5, 10.0, 0.0006, b"r_slice")
    gs = lib.FLETCHER_OpenSliceFile(*box, 12.5, 12.5, 10.0, 0.0006, b"g_slice")
    assert gs
    for f in frames:
        ref.DumpSliceFile(sx, sy, sz, fptr(f), rs)
        assert lib.FLETCHER_DumpSliceFile(sx, sy, sz, fptr(f), gs) == 0
    assert lib.FLETCHER_SliceFrames(gs) == 3
    ref.CloseSliceFile(rs)
    assert lib.FLETCHER_CloseSliceFile(gs) == 0
    rh, rd = files(tmp_path, "r_slice")
    gh, gd = files(tmp_path, "g_slice")
    assert gh == rh.replace(b"r_slice", b"g_slice")
    assert gd == rd


def test_slice_argument_errors(lib, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    lib.FLETCHER_ClearError()
    assert not lib.FLETCHER_OpenSliceFile(5, 4, 0, 1, 0, 1, 1.0, 1.0, 1.0, 1.0, b"bad")
    lib.FLETCHER_ClearError()
    s = lib.FLETCHER_OpenSliceFile(0, 20, 0, 1, 0, 1, 1.0, 1.0, 1.0, 1.0, b"big")
    a = np.zeros(10 * 10 * 10, np.float32)
    assert lib.FLETCHER_DumpSliceFile(10, 10, 10, fptr(a), s) != 0  # box beyond the array
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_CloseSliceFile(s) == 0
