"""Host logic of the batched path without a GPU: how BatchSolver hands its
members to the C-ABI (one sem2d_gpu_create_batch call for a list of
descriptions, sem2d_gpu_batch_add_many in groups for an iterator, the
members joining in the order given, the batch destroyed on an error), checked
against a stand-in for the library that records the calls; and the
argument checks of the batch entry points, which return before any CUDA
call."""
import ctypes as C

import pytest

from sem2dpack_gb300 import Sem2dError, abi, api
from sem2dpack_gb300._lib import lib


class FakeLib:
    """Records the batch calls; member i of a batch is the handle 1000 + i."""

    def __init__(self, fail_at=None):
        self.calls = []
        self.members = []
        self.fail_at = fail_at

    def sem2d_gpu_create_batch(self, arr, n, out):
        self.calls.append(("create_batch", [arr[i].npoin for i in range(n)]))
        self.members = [arr[i].npoin for i in range(n)]
        out._obj.value = 1
        return 0

    def sem2d_gpu_batch_open(self, out):
        self.calls.append(("open",))
        out._obj.value = 1
        return 0

    def sem2d_gpu_batch_add_many(self, h, arr, n):
        group = [arr[i].npoin for i in range(n)]
        self.calls.append(("add_many", group))
        if self.fail_at is not None and self.fail_at in group:
            return abi.SEM2D_E_ARG
        self.members.extend(group)
        return 0

    def sem2d_gpu_batch_close(self, h):
        self.calls.append(("close",))
        return 0

    def sem2d_gpu_batch_member(self, h, i):
        return 1000 + i

    def sem2d_gpu_destroy(self, h):
        self.calls.append(("destroy",))
        return 0

    def sem2d_gpu_last_error(self, h):
        return b"stand-in error"


def descs(n):
    out = []
    for i in range(n):
        d = abi.ProblemDesc()
        d.npoin = 10 + i  # identifies the member
        d.nt = 5
        out.append(d)
    return out


@pytest.fixture
def fake(monkeypatch):
    def make(**kw):
        f = FakeLib(**kw)
        monkeypatch.setattr(api, "lib", lambda: f)
        return f
    return make


def test_list_goes_through_one_create_batch(fake):
    f = fake()
    b = api.BatchSolver(descs(5))
    assert f.calls[0] == ("create_batch", [10, 11, 12, 13, 14])
    assert len(b) == 5 and [m.desc.npoin for m in b.members] == [10, 11, 12, 13, 14]
    assert b.nt == 5
    b.close()
    assert f.calls[-1] == ("destroy",)


def test_iterator_goes_in_groups_in_order(fake):
    f = fake()
    b = api.BatchSolver(iter(descs(7)), group=3)
    assert [c[0] for c in f.calls] == ["open", "add_many", "add_many", "add_many", "close"]
    assert [c[1] for c in f.calls if c[0] == "add_many"] == [[10, 11, 12], [13, 14, 15], [16]]
    assert f.members == list(range(10, 17))
    assert [m.desc.npoin for m in b.members] == list(range(10, 17))
    b.close()  # while the stand-in is in place
    assert f.calls[-1] == ("destroy",)


def test_failed_group_destroys_the_batch(fake):
    f = fake(fail_at=14)
    with pytest.raises(Sem2dError):
        api.BatchSolver(iter(descs(7)), group=3)
    assert ("close",) not in f.calls
    assert f.calls[-1] == ("destroy",)


def test_batch_entry_points_check_their_arguments():
    L = lib()
    h = C.c_void_p()
    assert L.sem2d_gpu_create_batch(None, 0, C.byref(h)) == abi.SEM2D_E_ARG
    arr = (abi.ProblemDesc * 1)()
    assert L.sem2d_gpu_create_batch(arr, 0, C.byref(h)) == abi.SEM2D_E_ARG
    assert L.sem2d_gpu_batch_add_many(None, arr, 1) == abi.SEM2D_E_ARG
