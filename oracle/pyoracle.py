"""ctypes binding of the ORACLE library (test infrastructure only).

Only the tests, the smoke check and the CPU-baseline leg of bench.py import
this module; the product never does.
"""
import ctypes as C
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(_HERE))

from sem2dpack_gb300 import abi  # noqa: E402
from oracle import build as _build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
        L.oc_setup_build.restype = vp
        L.oc_setup_build.argtypes = [C.POINTER(abi.Deck), C.c_char_p, C.c_int]
        L.oc_grid_build.restype = vp
        L.oc_grid_build.argtypes = [C.POINTER(abi.Deck), C.c_char_p, C.c_int]
        L.oc_setup_free.argtypes = [vp]
        L.oc_setup_sizes.argtypes = [vp, ip, ip, ip]
        L.oc_setup_ibool.argtypes = [vp, ip]
        L.oc_setup_coord.argtypes = [vp, dp]
        L.oc_setup_tags.argtypes = [vp, ip]
        L.oc_setup_knods.argtypes = [vp, ip]
        L.oc_setup_boundary.argtypes = [vp, C.c_int, ip]
        L.oc_setup_time.argtypes = [vp, dp, ip, dp]
        L.oc_setup_desc.argtypes = [vp, C.POINTER(abi.ProblemDesc)]
        L.oc_setup_rec_coord.argtypes = [vp, dp]
        L.oc_setup_fault_coord.argtypes = [vp, dp]
        L.oc_sim_create.restype = vp
        L.oc_sim_create.argtypes = [C.POINTER(abi.ProblemDesc), C.c_char_p, C.c_int]
        L.oc_sim_run.argtypes = [vp, C.c_int]
        L.oc_sim_step_count.argtypes = [vp]
        L.oc_sim_fields.argtypes = [vp, dp, dp, dp]
        L.oc_sim_seismograms.argtypes = [vp, dp]
        L.oc_sim_fault_series.argtypes = [vp, dp]
        L.oc_sim_fault_potency.argtypes = [vp, dp]
        L.oc_sim_strain_stress.argtypes = [vp, dp, dp]
        L.oc_sim_set_displacement.argtypes = [vp, dp]
        L.oc_sim_fault_state.argtypes = [vp, dp, dp, dp, dp, dp]
        L.oc_sim_free.argtypes = [vp]
        L.oc_gll_info.argtypes = [C.c_int, dp, dp, dp]
        L.oc_stf_eval.argtypes = [C.POINTER(abi.Stf), C.c_int, dp, dp]
        _lib = L
    return _lib


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def gll(n):
    x, w, H = np.zeros(n), np.zeros(n), np.zeros(n * n)
    lib().oc_gll_info(n, _p(x), _p(w), _p(H))
    return x, w, H.reshape(n, n, order="F")


class OracleSetup:
    """Restated init_main for a ParDeck (grid_only: mesh + spectral grid)."""

    def __init__(self, deck, grid_only=False):
        self.deck = deck
        self._c, self._keep = deck.to_c()
        err = C.create_string_buffer(512)
        fn = lib().oc_grid_build if grid_only else lib().oc_setup_build
        self.h = fn(C.byref(self._c), err, 512)
        if not self.h:
            raise RuntimeError("oracle setup failed: " + err.value.decode())
        ne, npn, ng = C.c_int(), C.c_int(), C.c_int()
        lib().oc_setup_sizes(self.h, C.byref(ne), C.byref(npn), C.byref(ng))
        self.nelem, self.npoin, self.ngll = ne.value, npn.value, ng.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().oc_setup_free(self.h)
            self.h = None

    def ibool(self):
        a = np.zeros(self.ngll * self.ngll * self.nelem, dtype=np.int32)
        lib().oc_setup_ibool(self.h, _p(a, C.c_int))
        return a.reshape(self.ngll, self.ngll, self.nelem, order="F")

    def coord(self):
        a = np.zeros(2 * self.npoin)
        lib().oc_setup_coord(self.h, _p(a))
        return a.reshape(2, self.npoin, order="F")

    def tags(self):
        a = np.zeros(self.nelem, dtype=np.int32)
        lib().oc_setup_tags(self.h, _p(a, C.c_int))
        return a

    def knods(self):
        a = np.zeros(4 * self.nelem, dtype=np.int32)
        lib().oc_setup_knods(self.h, _p(a, C.c_int))
        return a.reshape(4, self.nelem, order="F")

    def boundary(self, tag):
        n = lib().oc_setup_boundary(self.h, tag, None)
        a = np.zeros(max(n, 1), dtype=np.int32)
        lib().oc_setup_boundary(self.h, tag, _p(a, C.c_int))
        return a[:n]

    def time(self):
        dt, nt, cr = C.c_double(), C.c_int(), C.c_double()
        lib().oc_setup_time(self.h, C.byref(dt), C.byref(nt), C.byref(cr))
        return dt.value, nt.value, cr.value

    def rec_coord(self):
        n = lib().oc_setup_rec_coord(self.h, None)
        a = np.zeros(2 * max(n, 1))
        lib().oc_setup_rec_coord(self.h, _p(a))
        return a[: 2 * n].reshape(2, n, order="F")

    def fault_coord(self):
        n = lib().oc_setup_fault_coord(self.h, None)
        a = np.zeros(2 * max(n, 1))
        lib().oc_setup_fault_coord(self.h, _p(a))
        return a[: 2 * n].reshape(2, n, order="F")

    def desc(self):
        d = abi.ProblemDesc()
        lib().oc_setup_desc(self.h, C.byref(d))
        return d


class OracleSim:
    """Restated time loop driven by a ProblemDesc (the GPU library's input)."""

    def __init__(self, desc, owner=None):
        self._owner = owner  # keeps the arrays behind desc alive
        self.desc = desc
        err = C.create_string_buffer(512)
        self.h = lib().oc_sim_create(C.byref(desc), err, 512)
        if not self.h:
            raise RuntimeError("oracle sim failed: " + err.value.decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().oc_sim_free(self.h)
            self.h = None

    def run(self, nsteps):
        st = lib().oc_sim_run(self.h, nsteps)
        if st != 0:
            raise RuntimeError("oracle step failed with status %d" % st)

    @property
    def step(self):
        return lib().oc_sim_step_count(self.h)

    def fields(self):
        n = self.desc.npoin * self.desc.ndof
        d, v, a = np.zeros(n), np.zeros(n), np.zeros(n)
        lib().oc_sim_fields(self.h, _p(d), _p(v), _p(a))
        sh = (self.desc.npoin, self.desc.ndof)
        return d.reshape(sh, order="F"), v.reshape(sh, order="F"), a.reshape(sh, order="F")

    def seismograms(self):
        d = self.desc
        a = np.zeros(max(d.rec_nsamp * d.nrec * d.ndof, 1))
        lib().oc_sim_seismograms(self.h, _p(a))
        return a[: d.rec_nsamp * d.nrec * d.ndof].reshape(d.rec_nsamp, d.nrec, d.ndof, order="F")

    def fault_series(self):
        d = self.desc
        onx = (d.flt_oixn - d.flt_oix1) // max(d.flt_oixd, 1) + 1
        a = np.zeros(max(onx * 6 * d.flt_nsamp, 1))
        lib().oc_sim_fault_series(self.h, _p(a))
        return a[: onx * 6 * d.flt_nsamp].reshape(onx, 6, d.flt_nsamp, order="F")

    def set_displacement(self, d):
        a = np.asfortranarray(d, dtype=np.float64).reshape(-1, order="F")
        lib().oc_sim_set_displacement(self.h, _p(a))

    def strain_stress(self):
        d = self.desc
        sh = (d.ngll, d.ngll, d.ndof + 1, d.nelem)
        e, s = np.zeros(int(np.prod(sh))), np.zeros(int(np.prod(sh)))
        lib().oc_sim_strain_stress(self.h, _p(e), _p(s))
        return e.reshape(sh, order="F"), s.reshape(sh, order="F")

    def fault_potency(self):
        """(nt+1, 2, 3): potency of displacement and velocity at every step."""
        d = self.desc
        a = np.zeros(6 * (d.nt + 1))
        if d.nflt:
            lib().oc_sim_fault_potency(self.h, _p(a))
        return a.reshape(d.nt + 1, 2, 3)

    def fault_state(self):
        d = self.desc
        nf, nd = d.nflt, d.ndof
        D, V, T = np.zeros(nf * nd), np.zeros(nf * nd), np.zeros(2 * nf)
        MU, th = np.zeros(nf), np.zeros(nf)
        lib().oc_sim_fault_state(self.h, _p(D), _p(V), _p(T), _p(MU), _p(th))
        return (D.reshape(nf, nd, order="F"), V.reshape(nf, nd, order="F"),
                T.reshape(nf, 2, order="F"), MU, th)


def run_deck(deck, nsteps=None):
    """Build with the oracle, run nsteps (default: all) and return (setup, sim)."""
    s = OracleSetup(deck)
    sim = OracleSim(s.desc(), owner=s)
    sim.run(s.time()[1] if nsteps is None else nsteps)
    return s, sim


def rupture_time(v, dt, v_crit=1.0e-3):
    """Rupture time per node, restating the loop of the reference's
    post-processing (POST/python/post-process-fault.py:53-62) on a slip-rate
    array v[i, x] (sample i, node x): the first i in 0 .. nt-3 with
    v[i, x] < V_critical <= v[i+1, x] gives Rup_t[x] = i*dt; otherwise 0."""
    nt, nx = v.shape
    rup = np.zeros(nx)
    for x in range(nx):
        for i in range(nt - 2):
            if v[i, x] < v_crit and v[i + 1, x] >= v_crit:
                rup[x] = i * dt
                break
    return rup
