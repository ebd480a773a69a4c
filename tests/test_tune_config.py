"""Tile-shape configuration file (FLETCHER_TuneConfigStore / Lookup): the
line format of the reference's block-size tuner
(original_singleGPU_PDP/model.c:51-113, "%s | %d | %d | %d", appended) with
two extra fields; the batch tuner's candidate shapes and the batch API's
argument checks.  Host code only."""
import re

import numpy as np
import pytest


def test_store_then_lookup_and_reference_format(lib, tmp_path):
    import ctypes as C

    path = str(tmp_path / "configurations.txt").encode()
    # a line the reference's own tuner wrote: four fields, not ours
    with open(path, "w") as f:
        f.write("NVIDIA GB300 | 576 | 16 | 16\n")
    assert lib.FLETCHER_TuneConfigStore(path, b"NVIDIA GB300", 576, 0, 12, 5) == 0
    assert lib.FLETCHER_TuneConfigStore(path, b"NVIDIA GB300", 576, 2, 12, 4) == 0
    assert lib.FLETCHER_TuneConfigStore(path, b"Other GPU", 576, 0, 8, 5) == 0
    r, s = C.c_int(0), C.c_int(0)
    assert lib.FLETCHER_TuneConfigLookup(path, b"NVIDIA GB300", 576, 0, C.byref(r), C.byref(s)) == 1
    assert (r.value, s.value) == (12, 5)
    assert lib.FLETCHER_TuneConfigLookup(path, b"NVIDIA GB300", 576, 2, C.byref(r), C.byref(s)) == 1
    assert (r.value, s.value) == (12, 4)
    assert lib.FLETCHER_TuneConfigLookup(path, b"NVIDIA GB300", 200, 0, C.byref(r), C.byref(s)) == 0
    # the last matching line wins; shapes that are not built are skipped
    lib.FLETCHER_TuneConfigStore(path, b"NVIDIA GB300", 576, 0, 12, 6)
    lib.FLETCHER_TuneConfigStore(path, b"NVIDIA GB300", 576, 0, 7, 3)
    assert lib.FLETCHER_TuneConfigLookup(path, b"NVIDIA GB300", 576, 0, C.byref(r), C.byref(s)) == 1
    assert (r.value, s.value) == (12, 6)
    # every line still parses with the reference loader's leading fields
    ref = re.compile(r"^([^|]+) \| (-?\d+) \| (-?\d+) \| (-?\d+)")
    for line in open(path).read().splitlines():
        m = ref.match(line)
        assert m and m.group(1).strip() in ("NVIDIA GB300", "Other GPU")
        assert int(m.group(3)) * int(m.group(4)) <= 1024  # a valid block for the reference's kernel


def test_batch_tuner_candidates_are_built_shapes(lib, tmp_path):
    """Every (rows, stages) the batch tuner tries for a form is a built shape
    of that form's kernel: the configuration lookup accepts only those."""
    import ctypes as C

    from fletcher_petrobras_gb300.autotune import CANDIDATES, HALF_CANDIDATES

    r, s = C.c_int(0), C.c_int(0)
    for form, cands in ((0, CANDIDATES), (1, HALF_CANDIDATES), (2, HALF_CANDIDATES)):
        for rows, stages in cands:
            path = str(tmp_path / f"c{form}_{rows}_{stages}.txt").encode()
            assert lib.FLETCHER_TuneConfigStore(path, b"G", 100, form, rows, stages) == 0
            assert lib.FLETCHER_TuneConfigLookup(path, b"G", 100, form, C.byref(r), C.byref(s)) == 1, (form, rows, stages)
            assert (r.value, s.value) == (rows, stages)


def test_batch_form_is_checked_before_any_device_call(lib):
    from fletcher_petrobras_gb300._lib import fptr
    from fletcher_petrobras_gb300.batch import Batch

    with pytest.raises(ValueError):
        Batch(form="bf16")
    lib.FLETCHER_ClearError()
    assert lib.FLETCHER_BatchSetTileConfig(16, 5) != 0  # no batch yet
    lib.FLETCHER_ClearError()
    model = np.zeros(6 * 16 ** 3, np.float32)
    assert lib.FLETCHER_BatchAddShot(16, 16, 16, fptr(model), 8 + 16 * (8 + 16 * 8), 10) < 0  # no batch yet
    lib.FLETCHER_ClearError()
