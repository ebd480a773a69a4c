"""Tile-shape configuration file (FLETCHER_TuneConfigStore / Lookup): the
line format of the reference's block-size tuner
(original_singleGPU_PDP/model.c:51-113, "%s | %d | %d | %d", appended) with
two extra fields; host code only."""
import re


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
