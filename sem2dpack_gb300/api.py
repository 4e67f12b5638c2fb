"""Python API over the C-ABI: build a problem from a deck, run it on the GPU.

    from sem2dpack_gb300 import ParDeck, Problem, Solver
    prob = Problem(deck)            # host builder (init_main of the reference)
    sim = Solver(prob)              # upload to the GPU (sem2d_gpu_create)
    sim.step(prob.nt)               # the time loop (main.f90:51-96)
    sis = sim.seismograms()         # sis(nsamp, nrec, ndof)

There is no CPU execution path: Solver needs the compiled library and a
CUDA device and raises Sem2dError otherwise.
"""
import ctypes as C
import os
import time

import numpy as np

from . import abi
from ._lib import lib


class Sem2dError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("[%d] %s" % (code, msg))
        self.code = code


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def _host_check(st):
    if st != 0:
        raise Sem2dError(st, lib().sem2d_host_last_error().decode())


class Grid:
    """Mesh + spectral grid of a deck (sem2d_grid_build)."""

    def __init__(self, deck):
        self.deck = deck
        self._c, self._keep = deck.to_c()
        h = C.c_void_p()
        _host_check(lib().sem2d_grid_build(C.byref(self._c), C.byref(h)))
        self.h = h
        ne, npn, ng = C.c_int(), C.c_int(), C.c_int()
        lib().sem2d_grid_sizes(self.h, C.byref(ne), C.byref(npn), C.byref(ng))
        self.nelem, self.npoin, self.ngll = ne.value, npn.value, ng.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().sem2d_grid_destroy(self.h)
            self.h = None

    def ibool(self):
        a = np.zeros(self.ngll * self.ngll * self.nelem, dtype=np.int32)
        lib().sem2d_grid_ibool(self.h, _p(a, C.c_int))
        return a.reshape(self.ngll, self.ngll, self.nelem, order="F")

    def coord(self):
        a = np.zeros(2 * self.npoin)
        lib().sem2d_grid_coord(self.h, _p(a))
        return a.reshape(2, self.npoin, order="F")

    def tags(self):
        a = np.zeros(self.nelem, dtype=np.int32)
        lib().sem2d_grid_tags(self.h, _p(a, C.c_int))
        return a

    def boundary(self, tag):
        n = C.c_int()
        lib().sem2d_grid_boundary(self.h, tag, C.byref(n), None)
        a = np.zeros(max(n.value, 1), dtype=np.int32)
        lib().sem2d_grid_boundary(self.h, tag, C.byref(n), _p(a, C.c_int))
        return a[: n.value]

    def gll(self):
        n = self.ngll
        x, w, H = np.zeros(n), np.zeros(n), np.zeros(n * n)
        lib().sem2d_grid_gll(self.h, _p(x), _p(w), _p(H))
        return x, w, H.reshape(n, n, order="F")

    def fault_nodes(self, tags=None):
        """Fault node pairs as BC_DYNFLT_init forms them (bc_dynflt.f90:274-299)."""
        t1, t2 = tags or (self.deck.fault.tags if self.deck.fault else (5, 6))
        n1 = self.boundary(t1)
        if t2 <= 0:
            return n1, None
        n2 = self.boundary(t2)
        keep = n1 != n2
        return n1[keep], n2[keep]


class Problem:
    """Everything init_main builds (sem2d_problem_build) for one deck."""

    def __init__(self, deck, grid=None):
        self.deck = deck
        self.grid = grid if grid is not None else Grid(deck)
        self._c, self._keep = deck.to_c()
        h = C.c_void_p()
        _host_check(lib().sem2d_problem_build(self.grid.h, C.byref(self._c), C.byref(h)))
        self.h = h
        dt, nt, cr = C.c_double(), C.c_int(), C.c_double()
        lib().sem2d_problem_time(self.h, C.byref(dt), C.byref(nt), C.byref(cr))
        self.dt, self.nt, self.courant = dt.value, nt.value, cr.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().sem2d_problem_destroy(self.h)
            self.h = None

    def desc(self):
        d = abi.ProblemDesc()
        _host_check(lib().sem2d_problem_get_desc(self.h, C.byref(d)))
        return d

    def rec_coord(self):
        n = lib().sem2d_problem_rec_coord(self.h, None)
        a = np.zeros(2 * max(n, 1))
        lib().sem2d_problem_rec_coord(self.h, _p(a))
        return a[: 2 * n].reshape(2, n, order="F")

    def fault_coord(self):
        n = lib().sem2d_problem_fault_coord(self.h, None)
        a = np.zeros(2 * max(n, 1))
        lib().sem2d_problem_fault_coord(self.h, _p(a))
        return a[: 2 * n].reshape(2, n, order="F")


class Solver:
    """A problem resident on the GPU (sem2d_gpu_create ... destroy)."""

    def __init__(self, problem_or_desc, owner=None):
        if isinstance(problem_or_desc, Problem):
            self._owner = problem_or_desc
            self.desc = problem_or_desc.desc()
        else:
            self._owner = owner
            self.desc = problem_or_desc
        h = C.c_void_p()
        st = lib().sem2d_gpu_create(C.byref(self.desc), C.byref(h))
        if st != 0:
            raise Sem2dError(st, lib().sem2d_gpu_last_error(None).decode())
        self.h = h

    def _check(self, st):
        if st != 0:
            raise Sem2dError(st, lib().sem2d_gpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            lib().sem2d_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, nsteps):
        self._check(lib().sem2d_gpu_step(self.h, int(nsteps)))

    def step_timed(self, nsteps):
        """Like step(), with per-kernel CUDA-event timing; returns the summed
        milliseconds of (bulk, fault/counter, receiver) kernels."""
        ms = np.zeros(3)
        self._check(lib().sem2d_gpu_step_timed(self.h, int(nsteps), _p(ms)))
        return ms

    def run(self):
        """All remaining steps up to nt."""
        self.step(self.desc.nt - self.current_step)

    def sync(self):
        self._check(lib().sem2d_gpu_sync(self.h))

    def reset(self):
        self._check(lib().sem2d_gpu_reset(self.h))

    @property
    def stream(self):
        """The cudaStream_t (as an int) the solver launches on."""
        return lib().sem2d_gpu_stream(self.h)

    @property
    def current_step(self):
        return lib().sem2d_gpu_current_step(self.h)

    @property
    def launches(self):
        return lib().sem2d_gpu_kernel_launches(self.h)

    @property
    def tile(self):
        tx, tz = C.c_int(), C.c_int()
        self._check(lib().sem2d_gpu_tile_shape(self.h, C.byref(tx), C.byref(tz)))
        return tx.value, tz.value

    def fields(self, accel=False):
        n = self.desc.npoin * self.desc.ndof
        d, v = np.zeros(n), np.zeros(n)
        a = np.zeros(n) if accel else None
        self._check(lib().sem2d_gpu_get_fields(self.h, _p(d), _p(v), _p(a) if accel else None))
        sh = (self.desc.npoin, self.desc.ndof)
        out = [d.reshape(sh, order="F"), v.reshape(sh, order="F")]
        if accel:
            out.append(a.reshape(sh, order="F"))
        return tuple(out)

    def seismograms(self):
        d = self.desc
        n = d.rec_nsamp * d.nrec * d.ndof
        a = np.zeros(max(n, 1))
        self._check(lib().sem2d_gpu_get_seismograms(self.h, _p(a)))
        return a[:n].reshape(d.rec_nsamp, d.nrec, d.ndof, order="F")

    def fault_series(self):
        d = self.desc
        onx = (d.flt_oixn - d.flt_oix1) // max(d.flt_oixd, 1) + 1
        n = onx * 6 * d.flt_nsamp
        a = np.zeros(max(n, 1))
        self._check(lib().sem2d_gpu_get_fault(self.h, _p(a)))
        return a[:n].reshape(onx, 6, d.flt_nsamp, order="F")

    def strain_stress(self):
        """(strain, stress), each (ngll, ngll, ndof+1, nelem) in the
        reference's element order, from the current displacement."""
        d = self.desc
        n = d.ngll * d.ngll * (d.ndof + 1) * d.nelem
        e, s = np.zeros(n), np.zeros(n)
        self._check(lib().sem2d_gpu_get_strain_stress(self.h, _p(e), _p(s)))
        sh = (d.ngll, d.ngll, d.ndof + 1, d.nelem)
        return e.reshape(sh, order="F"), s.reshape(sh, order="F")

    def fault_potency(self):
        """(nt+1, 2, 3): potency of the displacement and of the velocity after
        every step (a handle created with desc.flt_potency = 1)."""
        a = np.zeros(6 * (self.desc.nt + 1))
        self._check(lib().sem2d_gpu_get_fault_potency(self.h, _p(a)))
        return a.reshape(self.desc.nt + 1, 2, 3)

    def fault_state(self):
        d = self.desc
        nf, nd = d.nflt, d.ndof
        D, V, T = np.zeros(nf * nd), np.zeros(nf * nd), np.zeros(2 * nf)
        MU, th = np.zeros(nf), np.zeros(nf)
        self._check(lib().sem2d_gpu_get_fault_state(self.h, _p(D), _p(V), _p(T), _p(MU), _p(th)))
        return (D.reshape(nf, nd, order="F"), V.reshape(nf, nd, order="F"),
                T.reshape(nf, 2, order="F"), MU, th)


class _Member(Solver):
    """Read access to one problem of a batch (outputs only; the batch steps,
    resets and destroys it)."""

    def __init__(self, batch, h, desc):
        self._owner = batch
        self.desc = desc
        self.h = h

    def close(self):
        self.h = None


class BatchSolver:
    """Independent problems advanced together by one launch per step.

    ``problems`` given as a list or tuple of problem descriptions
    (ProblemDesc, whose arrays the caller keeps alive through ``owners``)
    go through sem2d_gpu_create_batch.  Otherwise ``problems`` may be an
    iterator of Problems (or decks, or (deck, grid) pairs, or descriptions)
    taken ``group`` at a time (sem2d_gpu_batch_open / add_many / close):
    a group is built, uploaded and released before the next one, so host
    memory holds one group at a time.  Both calls set the members of a
    group up on several host threads.  ``batch[i]`` reads the outputs of
    problem i."""

    def __init__(self, problems, owners=None, group=None):
        self.h = None
        self._keep = list(owners or [])
        self.upload_seconds = 0.0  # time spent in the create / add / close calls
        if isinstance(problems, (list, tuple)) and problems and all(
                isinstance(p, abi.ProblemDesc) for p in problems):
            arr = (abi.ProblemDesc * len(problems))(*problems)
            h = C.c_void_p()
            t0 = time.perf_counter()
            st = lib().sem2d_gpu_create_batch(arr, len(problems), C.byref(h))
            self.upload_seconds = time.perf_counter() - t0
            if st != 0:
                raise Sem2dError(st, lib().sem2d_gpu_last_error(None).decode())
            self.h = h
            descs = [abi.ProblemDesc.from_buffer_copy(d) for d in problems]
        else:
            h = C.c_void_p()
            st = lib().sem2d_gpu_batch_open(C.byref(h))
            if st != 0:
                raise Sem2dError(st, lib().sem2d_gpu_last_error(None).decode())
            self.h = h
            descs = []
            env = os.environ.get("SEM2D_HOST_THREADS", "")
            group = group or (int(env) if env.isdigit() else 0) or min(16, os.cpu_count() or 1)
            held = []  # the group's problems, alive until their upload returns

            def flush():
                if not held:
                    return
                arr = (abi.ProblemDesc * len(held))(*[d for d, _ in held])
                t0 = time.perf_counter()
                self._check(lib().sem2d_gpu_batch_add_many(h, arr, len(held)))
                self.upload_seconds += time.perf_counter() - t0
                # only the sizes of the descriptions are used from now on
                descs.extend(abi.ProblemDesc.from_buffer_copy(d) for d, _ in held)
                held.clear()

            try:
                for p in problems:
                    if isinstance(p, abi.ProblemDesc):
                        d = p
                    else:
                        if not isinstance(p, Problem):
                            p = Problem(*p) if isinstance(p, tuple) else Problem(p)
                        d = p.desc()
                    held.append((d, p))
                    del p
                    if len(held) >= group:
                        flush()
                flush()
                t0 = time.perf_counter()
                self._check(lib().sem2d_gpu_batch_close(h))
                self.upload_seconds += time.perf_counter() - t0
            except Exception:
                self.close()
                raise
        self.members = [_Member(self, C.c_void_p(lib().sem2d_gpu_batch_member(h, i)), descs[i])
                        for i in range(len(descs))]
        self.nt = descs[0].nt

    def _check(self, st):
        if st != 0:
            raise Sem2dError(st, lib().sem2d_gpu_last_error(self.h).decode())

    def __len__(self):
        return len(self.members)

    def __getitem__(self, i):
        return self.members[i]

    def close(self):
        if getattr(self, "h", None):
            for m in getattr(self, "members", []):
                m.h = None
            lib().sem2d_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, nsteps):
        self._check(lib().sem2d_gpu_step(self.h, int(nsteps)))

    def step_timed(self, nsteps):
        ms = np.zeros(3)
        self._check(lib().sem2d_gpu_step_timed(self.h, int(nsteps), _p(ms)))
        return ms

    def run(self):
        self.step(self.nt - self.current_step)

    def sync(self):
        self._check(lib().sem2d_gpu_sync(self.h))

    def reset(self):
        self._check(lib().sem2d_gpu_reset(self.h))

    @property
    def stream(self):
        return lib().sem2d_gpu_stream(self.h)

    @property
    def current_step(self):
        return lib().sem2d_gpu_current_step(self.h)

    @property
    def launches(self):
        return lib().sem2d_gpu_kernel_launches(self.h)

    @property
    def tile(self):
        tx, tz = C.c_int(), C.c_int()
        self._check(lib().sem2d_gpu_tile_shape(self.h, C.byref(tx), C.byref(tz)))
        return tx.value, tz.value
