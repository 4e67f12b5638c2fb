"""The tuning cache and the selection rule of the march kernels' launch
shape (autotune.cpp), on the CPU: keys, record/lookup round trips, the
file format, and the choice among timed candidates."""
import ctypes as C
import json

from sem2dpack_gb300 import _lib, abi


def key(ndof, mat, nodes, members, nsm):
    buf = C.create_string_buffer(160)
    assert _lib.lib().sem2d_tune_key(ndof, mat, nodes, members, nsm, buf, 160) == 0
    return buf.value


def entry(cz, warps, ms):
    return abi.TuneEntry(cz, warps, ms)


def test_keys_bucket_by_powers_of_two():
    assert key(2, 2, 423475640, 256, 152) == b"march ndof=2 mat=2 nodes=2^28 members=2^8 sm=152"
    assert key(2, 2, 300000000, 300, 152) == key(2, 2, 423475640, 256, 152)
    assert key(2, 2, 423475640, 200, 152) != key(2, 2, 423475640, 256, 152)
    assert key(1, 2, 1284002, 0, 152) == b"march ndof=1 mat=2 nodes=2^20 members=2^0 sm=152"
    assert key(1, 2, 1284002, 0, 148) != key(1, 2, 1284002, 0, 152)
    assert key(2, 0, 1284002, 0, 152) != key(2, 2, 1284002, 0, 152)
    buf = C.create_string_buffer(8)
    assert _lib.lib().sem2d_tune_key(2, 2, 1000, 0, 152, buf, 8) == abi.SEM2D_E_ARG  # too short
    assert _lib.lib().sem2d_tune_key(3, 2, 1000, 0, 152, C.create_string_buffer(160), 160) == abi.SEM2D_E_ARG


def test_record_and_lookup(tmp_path):
    L = _lib.lib()
    path = str(tmp_path / "sub" / "tune.json").encode()
    k1, k2 = key(2, 2, 1 << 20, 0, 152), key(1, 2, 1 << 20, 0, 152)
    out = abi.TuneEntry()
    assert L.sem2d_tune_lookup(path, k1, C.byref(out)) == 0  # no file yet
    assert L.sem2d_tune_record(path, k1, C.byref(entry(32, 1, 4.5))) == 0
    assert L.sem2d_tune_record(path, k2, C.byref(entry(16, 4, 0.02))) == 0
    assert L.sem2d_tune_lookup(path, k1, C.byref(out)) == 1
    assert (out.chunk_rows, out.warps_per_cta) == (32, 1)
    assert abs(out.ms_per_step - 4.5) < 1e-9
    # a new record replaces the old one
    assert L.sem2d_tune_record(path, k1, C.byref(entry(8, 4, 3.0))) == 0
    assert L.sem2d_tune_lookup(path, k1, C.byref(out)) == 1
    assert (out.chunk_rows, out.warps_per_cta) == (8, 4)
    lines = (tmp_path / "sub" / "tune.json").read_text().splitlines()
    assert len(lines) == 2
    recs = {json.loads(x)["key"]: json.loads(x) for x in lines}
    assert recs[k1.decode()]["chunk_rows"] == 8 and recs[k2.decode()]["warps_per_cta"] == 4
    # unreadable lines are skipped, the others still read
    with open(path, "a") as f:
        f.write('{"key": "broken", "chunk_rows": \n')
        f.write('{"key": "bad warps", "chunk_rows": 4, "warps_per_cta": 3, "ms_per_step": 1}\n')
    assert L.sem2d_tune_lookup(path, k2, C.byref(out)) == 1
    assert L.sem2d_tune_lookup(path, b"bad warps", C.byref(out)) == 0
    assert L.sem2d_tune_record(path, b'quote"inside', C.byref(entry(1, 1, 1.0))) == abi.SEM2D_E_ARG


def test_selection_keeps_the_default_within_the_margin():
    L = _lib.lib()
    arr = (abi.TuneEntry * 4)(entry(16, 4, 1.00), entry(16, 1, 0.99), entry(32, 4, 1.20), entry(8, 4, 0.0))
    assert L.sem2d_tune_select(arr, 4, 0.02) == 0  # 1 % faster: noise
    arr[1].ms_per_step = 0.95
    assert L.sem2d_tune_select(arr, 4, 0.02) == 1  # 5 % faster
    arr[2].ms_per_step = 0.90
    assert L.sem2d_tune_select(arr, 4, 0.02) == 2
    assert L.sem2d_tune_select(arr, 4, 0.0) == 2
    assert L.sem2d_tune_select(arr, 0, 0.02) == abi.SEM2D_E_ARG


def test_cache_path_from_the_environment(monkeypatch, tmp_path):
    L = _lib.lib()
    monkeypatch.setenv("SEM2D_TUNE_CACHE", str(tmp_path / "x.json"))
    need = L.sem2d_tune_cache_path(None, 0)
    assert need == len(str(tmp_path / "x.json")) + 1
    buf = C.create_string_buffer(need)
    assert L.sem2d_tune_cache_path(buf, need) == 0
    assert buf.value.decode() == str(tmp_path / "x.json")
    monkeypatch.delenv("SEM2D_TUNE_CACHE")
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    buf = C.create_string_buffer(1024)
    assert L.sem2d_tune_cache_path(buf, 1024) == 0
    assert buf.value.decode() == str(tmp_path / "sem2dpack_gb300" / "tune.json")
