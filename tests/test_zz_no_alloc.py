"""sem2d_gpu_step_noalloc: the time step on caller-owned device memory.

Callers that cannot call cudaMalloc -- for instance code whose device
memory all belongs to another framework's pool -- hand the library their
own arrays in the documented lattice layout.  This test is such a caller:
every device array is a torch tensor, built from the problem descriptor by
the layout rules in include/sem2d_gpu.h, and the result of two calls in a
row is compared with the handle-based entry point (sem2d_gpu_create /
sem2d_gpu_step) on the same problem.  The file is named to be collected
last, so a run that stops at the first failure has run everything else.
"""
import ctypes as C
import math

import numpy as np
import pytest

from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Solver, abi, workloads
from sem2dpack_gb300._lib import lib

pytestmark = pytest.mark.gpu

TOL = {PRECISION_FP64: 1e-10, PRECISION_MIXED: 1e-4}


def _arr(d, name, n, dtype=np.float64):
    return np.ctypeslib.as_array(getattr(d, name), shape=(n,)).astype(dtype)


def lattice_arrays(d):
    """Lattice layout of a problem without fault, from the descriptor."""
    N, ne, npn, nd = d.ngll, d.nelem, d.npoin, d.ndof
    ib = _arr(d, "ibool", N * N * ne, np.int64).reshape(N, N, ne, order="F") - 1
    xy = _arr(d, "coord", 2 * npn).reshape(2, npn, order="F")
    x0, z0 = xy[0, ib[0, 0]], xy[1, ib[0, 0]]
    x1, z1 = xy[0, ib[N - 1, N - 1]], xy[1, ib[N - 1, N - 1]]
    xs, zs = np.unique(x0), np.unique(z0)
    nx, nz = xs.size, zs.size
    ex, ez = np.searchsorted(xs, x0), np.searchsorted(zs, z0)
    row0 = np.append(np.arange(nz) * (N - 1), nz * (N - 1) + 1).astype(np.int32)
    LX, LZ = nx * (N - 1) + 1, int(row0[-1])
    pitch = (LX + 7) // 8 * 8
    plane = pitch * LZ
    g2l = np.empty(npn, dtype=np.int64)
    ii, jj = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    lat = ((row0[ez][None, None, :] + jj[:, :, None]) * pitch + ex[None, None, :] * (N - 1) + ii[:, :, None])
    g2l[ib.ravel()] = lat.ravel()
    la, mu = _arr(d, "la", N * N * ne), _arr(d, "mu", N * N * ne)
    mat = [np.zeros(plane), np.zeros(plane)]
    mat[0][g2l[ib.ravel(order="F")]] = la
    mat[1][g2l[ib.ravel(order="F")]] = mu
    rm = _arr(d, "rmass", npn * nd).reshape(npn, nd, order="F")
    rmass = np.ones(plane)
    rmass[g2l] = rm[:, 0]
    I, J = g2l % pitch, g2l // pitch
    nslot = 2 * LX + 2 * (LZ - 2)

    def slot(I, J):
        if J == 0:
            return I
        if J == LZ - 1:
            return LX + I
        if I == 0:
            return 2 * LX + J - 1
        if I == LX - 1:
            return 2 * LX + LZ - 2 + J - 1
        return -1

    per_rm, per_ca, per_cb = np.zeros(nd * nslot), np.zeros(nd * nslot), np.zeros(nd * nslot)
    for p in range(npn):
        s = slot(I[p], J[p])
        if s >= 0:
            per_rm[np.arange(nd) * nslot + s] = rm[p]
    abs_node = _arr(d, "abs_node", d.nabs, np.int64) - 1
    abs_c = _arr(d, "abs_C", d.nabs * nd).reshape(d.nabs, nd, order="F")
    used = np.zeros(nslot, dtype=int)
    for k, p in enumerate(abs_node):
        s = slot(I[p], J[p])
        dst = per_ca if used[s] == 0 else per_cb
        dst[np.arange(nd) * nslot + s] = abs_c[k]
        used[s] += 1
    dxdxi, dzdeta = np.zeros(nx), np.zeros(nz)
    dxdxi[ex], dzdeta[ez] = 0.5 * (x1 - x0), 0.5 * (z1 - z0)
    src = _arr(d, "src_node", d.nsrc, np.int64) - 1
    amp = np.zeros((d.nsrc, nd, d.nt + 1))
    for s in range(d.nsrc):
        f0, t0, a0 = d.src_f0[s], d.src_t0[s], d.src_ampli[s]
        rel, td = d.src_relamp[s], d.src_tdelay[s]
        for it in range(1, d.nt + 1):
            arg = 3.141592653589793 * f0 * (it * d.dt - td - t0)
            arg = arg * arg
            a = -((a0 * (1.0 - 2.0 * arg)) * math.exp(-arg)) * rel
            amp[s, :, it] = a if nd == 1 else [d.src_dir[2 * s] * a, d.src_dir[2 * s + 1] * a]
    return dict(N=N, nd=nd, nx=nx, nz=nz, LX=LX, LZ=LZ, pitch=pitch, plane=plane, g2l=g2l,
                row0=row0, mat=mat, rmass=rmass, per_rm=per_rm, per_ca=per_ca, per_cb=per_cb,
                xix=1.0 / dxdxi, etaz=1.0 / dzdeta, dxdxi=dxdxi, dzdeta=dzdeta,
                src_I=I[src].astype(np.int32), src_J=J[src].astype(np.int32), src_amp=amp.ravel())


def make_args(d, L, torch, precision):
    real = torch.float32 if precision == PRECISION_MIXED else torch.float64
    dev = {}

    def put(name, a, dtype=None):
        dev[name] = torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)
        return C.c_void_p(dev[name].data_ptr())

    args = abi.LatticeArgs()
    args.ngll, args.ndof, args.precision = L["N"], L["nd"], precision
    args.nx, args.nz, args.LX, args.LZ, args.pitch = L["nx"], L["nz"], L["LX"], L["LZ"], L["pitch"]
    args.row0 = put("row0", L["row0"], torch.int32)
    args.hprime, args.wgll = d.hprime, d.wgll
    args.d = put("d", np.zeros(L["nd"] * L["plane"]), real)
    args.v = put("v", np.zeros(L["nd"] * L["plane"]), real)
    args.rmass = put("rmass", L["rmass"], real)
    args.per_rm = put("per_rm", L["per_rm"], real)
    args.per_Ca = put("per_ca", L["per_ca"], real)
    args.per_Cb = put("per_cb", L["per_cb"], real)
    args.mat_iso = 1
    args.mat[0] = put("la", L["mat"][0], real)
    args.mat[1] = put("mu", L["mat"][1], real)
    args.xix = put("xix", L["xix"], real)
    args.etaz = put("etaz", L["etaz"], real)
    args.dxdxi = put("dxdxi", L["dxdxi"], real)
    args.dzdeta = put("dzdeta", L["dzdeta"], real)
    args.nsrc = d.nsrc
    args.src_I = put("src_I", L["src_I"], torch.int32)
    args.src_J = put("src_J", L["src_J"], torch.int32)
    args.src_amp = put("src_amp", L["src_amp"], torch.float64)
    args.nt, args.step0, args.dt, args.kd2_form = d.nt, 0, d.dt, d.kd2_form
    return args, dev


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_noalloc_matches_handle_path(precision):
    torch = pytest.importorskip("torch")
    P = workloads.build(workloads.plain_psv(scale=0.2, nsteps=120))
    d = P.desc()
    d.precision = precision
    ref = Solver(d, owner=P)
    ref.step(50)
    ref.step(70)
    d_ref, v_ref = ref.fields()
    L = lattice_arrays(d)
    args, dev = make_args(d, L, torch, precision)
    assert lib().sem2d_gpu_step_noalloc(C.byref(args), 50, None) == 0
    args.step0 = 50
    assert lib().sem2d_gpu_step_noalloc(C.byref(args), 70, None) == 0
    torch.cuda.synchronize()
    nd, plane, g2l = L["nd"], L["plane"], L["g2l"]
    v = dev["v"].double().cpu().numpy().reshape(nd, plane)[:, g2l].T
    dn = dev["d"].double().cpu().numpy().reshape(nd, plane)[:, g2l].T
    rel = np.linalg.norm(v - v_ref) / np.linalg.norm(v_ref)
    assert rel <= TOL[precision]
    # the state is the displacement of the next step: displ + dt*veloc
    pred = d_ref + d.dt * v_ref
    assert np.linalg.norm(dn - pred) / np.linalg.norm(pred) <= TOL[precision]


def test_noalloc_reports_device_failures_through_status(monkeypatch):
    """A step whose bounded wait runs out (no polls allowed: SEM2D_SPIN_LIMIT
    = 0) stores SEM2D_E_TIMEOUT in the caller's status int; the library
    never clears it, and a later call with the normal limit leaves it set
    until the caller resets it."""
    torch = pytest.importorskip("torch")
    P = workloads.build(workloads.plain_psv(scale=0.2, nsteps=20))
    d = P.desc()
    d.precision = PRECISION_FP64
    L = lattice_arrays(d)
    args, dev = make_args(d, L, torch, PRECISION_FP64)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    args.status = C.c_void_p(status.data_ptr())
    monkeypatch.setenv("SEM2D_SPIN_LIMIT", "0")
    assert lib().sem2d_gpu_step_noalloc(C.byref(args), 2, None) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == abi.SEM2D_E_TIMEOUT
    monkeypatch.delenv("SEM2D_SPIN_LIMIT")
    args.step0 = 0
    assert lib().sem2d_gpu_step_noalloc(C.byref(args), 2, None) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == abi.SEM2D_E_TIMEOUT  # sticky
    status.zero_()
    dev["d"].zero_()
    dev["v"].zero_()
    assert lib().sem2d_gpu_step_noalloc(C.byref(args), 2, None) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0


def test_noalloc_rejects_oversized_problems():
    """Partner buffers beyond SEM2D_NOALLOC_SCRATCH_BYTES are refused before
    any device work."""
    args = abi.LatticeArgs()
    args.ngll, args.ndof, args.precision = 5, 2, PRECISION_FP64
    args.nx, args.nz = 1000, 1000
    args.LX, args.LZ, args.pitch = 4001, 4001, 4008
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    for f in ("row0", "d", "v", "rmass", "per_rm", "per_Ca", "per_Cb", "xix", "etaz", "dxdxi", "dzdeta"):
        setattr(args, f, dummy)
    args.mat[0] = dummy
    w = (C.c_double * 25)()
    args.hprime, args.wgll = C.cast(w, abi.P_double), C.cast(w, abi.P_double)
    args.nt = 10
    assert lib().sem2d_gpu_step_noalloc(C.byref(args), 1, None) == abi.SEM2D_E_ARG
    assert b"too large" in lib().sem2d_gpu_last_error(None)
