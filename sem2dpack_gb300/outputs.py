"""Output files in the reference's formats, so that its readers (the
JUPYTER/POST scripts of SEM2DPACK, Seismic Unix) read a GPU run unchanged.

  seismograms   Ux_sem2d.dat, Uz_sem2d.dat (P-SV) or Uy_sem2d.dat (SH):
                direct-access FP32, record k = the nsamp samples of
                receiver k (REC_write, receivers.f90:351-392);
                SeisHeader_sem2d.hdr: 'DT NSAMP NSTA', values, 'XSTA ZSTA',
                one coordinate pair per receiver (REC_init, receivers.f90:
                212-221)
  fault         FltXX_sem2d.dat: Fortran unformatted sequential, per output
                time 6 records of NPTS FP32 values (slip, slip rate, shear
                and normal stress, friction coefficient, T_stick), each
                record framed by its 4-byte byte count (BC_DYNFLT_write,
                bc_dynflt.f90:751-778); FltXX_sem2d.hdr (NPTS NDAT NSAMP
                DELT, field names, node coordinates) and FltXX_sem2d.csh
                (bc_dynflt.f90:455-518)
  potency       FltXX_potency_sem2d.tab: one line per step, 6D24.16 (P-SV:
                potency of d then v, 3 values each; SH: 2 each)
                (bc_dynflt.f90:436,757)
  fault init    FltXX_init_sem2d.tab: T0 shear, T0 normal, mu, B per output
                node (bc_dynflt.f90:446-452)
  grid          grid_sem2d.hdr: 'NELEM  NPGEO  NGNOD  NPOIN  NGLL', values
                (SE_init, spec_grid.f90:136-141); ibool_sem2d.dat: direct
                access, record e = the NGLL x NGLL global node numbers of
                element e, int32, 1-based (SE_init_numbering,
                spec_grid.f90:298-307); coord_sem2d.dat: direct access,
                record i = (x, z) of node i in FP32 (SE_init_coord,
                spec_grid.f90:363-371)
  snapshots     {d,v,a}{x,z|y}_NNN_sem2d.dat: the node field in FP32, node
                order (PLOT_FIELD, plot_gen.f90:180-214; IO_rw_field,
                stdio.f90:113-139); e11/e22/e12 (SH e13/e23) and s11/s22/s12
                (SH s13/s23)_NNN_sem2d.dat: direct access, record e = the
                NGLL x NGLL values of element e in FP32 (plot_gen.f90:
                220-300); div/curl_NNN_sem2d.dat: divergence and curl
                of the velocity (P-SV), same records.  NNN = (it - it1) /
                itd, three digits

Values are written little-endian, as the reference built with gfortran on
x86 or Arm writes them.
"""
import os

import numpy as np

__all__ = ["write_seismograms", "read_seismograms", "write_fault", "read_fault", "write_potency", "write_run",
           "write_fault_init", "write_grid", "read_grid", "write_snapshot", "rupture_time"]

V_CRITICAL = 1.0e-3  # slip rate (m/s) that marks rupture (post-process-fault.py:53)


def rupture_time(slip_rate, odt, v_crit=V_CRITICAL):
    """Rupture time of every fault node from its slip-rate series.

    slip_rate is (onx, nsamp), the second record of the fault series
    (Solver.fault_series()[:, 1, :]) sampled every odt seconds.  The
    reference's post-processing (POST/python/post-process-fault.py:55-62)
    takes, per node, the first sample i (i = 0 .. nsamp-3) with v[i] < v_crit
    and v[i+1] >= v_crit and returns i*odt; a node whose slip rate never
    crosses v_crit gets 0.  Returns (times (onx,), sample index (onx,), with
    -1 where there is no crossing).
    """
    v = np.asarray(slip_rate, dtype=np.float64)
    onx, ns = v.shape
    if ns < 3:
        return np.zeros(onx), np.full(onx, -1, dtype=np.int64)
    cross = (v[:, : ns - 2] < v_crit) & (v[:, 1: ns - 1] >= v_crit)
    hit = cross.any(axis=1)
    idx = np.where(hit, np.argmax(cross, axis=1), -1).astype(np.int64)
    return np.where(hit, idx * float(odt), 0.0), idx


def _fmt_list(*vals):
    """Fortran list-directed style line: values separated by blanks."""
    out = []
    for v in vals:
        if isinstance(v, (int, np.integer)):
            out.append("%12d" % int(v))
        else:
            out.append("%25.16E" % float(v))
    return " " + " ".join(out)


def write_seismograms(path, sis, tsamp, coords):
    """sis (nsamp, nrec, ndof) as Solver.seismograms() returns it; tsamp the
    sampling interval (isamp * dt); coords (2, nrec) receiver positions."""
    sis = np.asarray(sis)
    nsamp, nrec, ndof = sis.shape
    os.makedirs(path, exist_ok=True)
    names = ["Uy"] if ndof == 1 else ["Ux", "Uz"]
    for c, name in enumerate(names):
        data = np.ascontiguousarray(sis[:, :, c].T, dtype="<f4")  # record k = receiver k
        data.tofile(os.path.join(path, name + "_sem2d.dat"))
    with open(os.path.join(path, "SeisHeader_sem2d.hdr"), "w") as f:
        f.write(" DT NSAMP NSTA\n")
        f.write(_fmt_list(np.float32(tsamp), nsamp, nrec) + "\n")
        f.write(" XSTA ZSTA\n")
        for k in range(nrec):
            f.write(_fmt_list(coords[0][k], coords[1][k]) + "\n")


def read_seismograms(path, ndof):
    """(sis (nsamp, nrec, ndof), tsamp, coords (2, nrec)) from a folder
    written by the reference or by write_seismograms."""
    with open(os.path.join(path, "SeisHeader_sem2d.hdr")) as f:
        lines = f.read().split("\n")
    dt, nsamp, nrec = lines[1].split()
    nsamp, nrec = int(nsamp), int(nrec)
    coords = np.array([[float(v) for v in lines[3 + k].split()] for k in range(nrec)]).T
    names = ["Uy"] if ndof == 1 else ["Ux", "Uz"]
    sis = np.zeros((nsamp, nrec, ndof))
    for c, name in enumerate(names):
        a = np.fromfile(os.path.join(path, name + "_sem2d.dat"), dtype="<f4")
        sis[:, :, c] = a.reshape(nrec, nsamp).T
    return sis, float(dt), coords


def _record(f, values):
    data = np.ascontiguousarray(values, dtype="<f4").tobytes()
    n = np.array([len(data)], dtype="<i4").tobytes()
    f.write(n + data + n)


FAULT_FIELDS = "Slip:Slip_Rate:Shear_Stress:Normal_Stress:Friction:T_stick"


def write_fault(path, tag, series, odt, coords):
    """series (onx, 6, nsamp) as Solver.fault_series() returns it; odt the
    output interval (oitd * dt); coords (2, onx) of the output nodes."""
    series = np.asarray(series)
    onx, ndat, nsamp = series.shape
    os.makedirs(path, exist_ok=True)
    name = os.path.join(path, "Flt%02d_sem2d" % int(tag))
    with open(name + ".dat", "wb") as f:
        for s in range(nsamp):
            for q in range(ndat):
                _record(f, series[:, q, s])
    with open(name + ".hdr", "w") as f:
        f.write(" NPTS NDAT NSAMP DELT\n")
        f.write(_fmt_list(onx, ndat, nsamp, odt) + "\n")
        f.write(" " + FAULT_FIELDS + "\n")
        f.write(" XPTS ZPTS\n")
        for k in range(onx):
            f.write(_fmt_list(coords[0][k], coords[1][k]) + "\n")
    base = os.path.basename(name)
    with open(name + ".csh", "w") as f:
        f.write(" #!/bin/csh -f\n")
        f.write(" #USAGE: %s.csh node field\n" % base)
        f.write(" @ ifs = $2 - 1\n")
        f.write("subset <%s.dat n1=%d n2=%d n3=%d ix1s=$1 ix2s=$ifs | b2a n1=1 > %s.$1.$ifs.tab\n"
                % (base, onx + 2, ndat, nsamp, base))


def read_fault(path, tag):
    """(series (onx, ndat, nsamp), odt, coords (2, onx)) of FltXX_sem2d.*"""
    name = os.path.join(path, "Flt%02d_sem2d" % int(tag))
    with open(name + ".hdr") as f:
        lines = f.read().split("\n")
    onx, ndat, nsamp, odt = lines[1].split()
    onx, ndat, nsamp = int(onx), int(ndat), int(nsamp)
    coords = np.array([[float(v) for v in lines[4 + k].split()] for k in range(onx)]).T
    raw = np.fromfile(name + ".dat", dtype="<f4").reshape(nsamp, ndat, onx + 2)
    head = raw[:, :, 0].view("<i4")
    if np.any(head != 4 * onx):
        raise ValueError("record markers do not match NPTS")
    return np.transpose(raw[:, :, 1:-1], (2, 1, 0)).astype(np.float64), float(odt), coords


def write_potency(path, tag, potency, ndof):
    """potency (nt+1, 2, 3) as Solver.fault_potency() returns it."""
    os.makedirs(path, exist_ok=True)
    k = 3 if ndof == 2 else 2
    with open(os.path.join(path, "Flt%02d_potency_sem2d.tab" % int(tag)), "w") as f:
        for row in np.asarray(potency):
            vals = list(row[0][:k]) + list(row[1][:k])
            f.write("".join(("%24.16E" % v).replace("E", "D") for v in vals) + "\n")


def write_fault_init(path, tag, T0, mu, B):
    """T0 (onx, 2) initial shear and normal stress, mu (onx) initial friction
    coefficient, B (onx) boundary weights of the output nodes."""
    os.makedirs(path, exist_ok=True)
    with open(os.path.join(path, "Flt%02d_init_sem2d.tab" % int(tag)), "w") as f:
        for k in range(len(mu)):
            f.write(_fmt_list(T0[k][0], T0[k][1], mu[k], B[k]) + "\n")


def write_grid(path, grid):
    """grid_sem2d.hdr, ibool_sem2d.dat and coord_sem2d.dat of a Grid.  The
    Cartesian mesher's geometric nodes are the (nx+1) x (nz+1) element
    corners, one row more when a fault splits the mesh (nzp,
    mesh_cartesian.f90:233-240), 4 per element."""
    os.makedirs(path, exist_ok=True)
    deck = grid.deck
    nx, nz = deck.nelem
    split = deck.ezflt > 0 or (deck.ezflt == -1 and nz // 2 > 0)
    npgeo = (nx + 1) * (nz + (2 if split else 1))
    with open(os.path.join(path, "grid_sem2d.hdr"), "w") as f:
        f.write(" NELEM  NPGEO  NGNOD  NPOIN  NGLL\n")
        f.write(_fmt_list(grid.nelem, npgeo, 4, grid.npoin, grid.ngll) + "\n")
    ib = grid.ibool()  # (ngll, ngll, nelem), 1-based
    np.ascontiguousarray(np.transpose(ib, (2, 1, 0)), dtype="<i4").tofile(os.path.join(path, "ibool_sem2d.dat"))
    xz = grid.coord()  # (2, npoin)
    np.ascontiguousarray(xz.T, dtype="<f4").tofile(os.path.join(path, "coord_sem2d.dat"))


def read_grid(path):
    """(sizes dict, ibool (ngll, ngll, nelem) 1-based, coord (2, npoin)
    FP32) from grid_sem2d.hdr / ibool_sem2d.dat / coord_sem2d.dat."""
    with open(os.path.join(path, "grid_sem2d.hdr")) as f:
        lines = f.read().split("\n")
    keys = lines[0].split()
    sizes = dict(zip(keys, (int(v) for v in lines[1].split())))
    n, ne, npn = sizes["NGLL"], sizes["NELEM"], sizes["NPOIN"]
    ib = np.fromfile(os.path.join(path, "ibool_sem2d.dat"), dtype="<i4").reshape(ne, n, n)
    xz = np.fromfile(os.path.join(path, "coord_sem2d.dat"), dtype="<f4").reshape(npn, 2)
    return sizes, np.transpose(ib, (2, 1, 0)), xz.T


def write_snapshot(path, solver, index, fields="V", grid=None):
    """The binary snapshot files of one output time for the SNAP_DEF
    `fields` letters D, V, A (node fields), E (strain) and S (stress);
    `index` is the NNN of the file names; A needs a handle that keeps the
    accelerations (Newmark, HHT-alpha or 'A' receivers).  S of a
    Kelvin-Voigt material is the stress of d + eta v, as the reference's
    (MAT_stress_dv, mat_gen.f90:626-641).  The divergence and curl of the
    velocity (d, c; MAT_divcurl_PSV, mat_gen.f90:802-825) need the Grid of
    a P-SV problem and are skipped for SH, as the reference skips them."""
    d = solver.desc
    fields = str(fields)
    bad = set(fields) - set("DVAESdc")
    if bad:
        raise ValueError("snapshot fields %s are not written" % sorted(bad))
    os.makedirs(path, exist_ok=True)
    tag = "%03d" % int(index)
    comps = ["y"] if d.ndof == 1 else ["x", "z"]
    want = [c for c in "DVA" if c in fields]
    if want:
        got = solver.fields(accel="A" in want)
        byname = {"D": got[0], "V": got[1]}
        if "A" in want:
            byname["A"] = got[2]
        for c in want:
            for k, comp in enumerate(comps):
                np.ascontiguousarray(byname[c][:, k], dtype="<f4").tofile(
                    os.path.join(path, "%s%s_%s_sem2d.dat" % (c.lower(), comp, tag)))
    if ("d" in fields or "c" in fields) and d.ndof == 2:
        # an SH problem has no divergence or curl: the reference drops them
        # (plot_gen.f90:100), and so does this writer
        if grid is None:
            raise ValueError("div/curl snapshots of a P-SV problem need its Grid")
        _write_divcurl(path, tag, solver.fields()[1], grid, fields)
    if "E" in fields or "S" in fields:
        strain, stress = solver.strain_stress()  # (ngll, ngll, ndof+1, nelem)
        names = (("13", "23") if d.ndof == 1 else ("11", "22", "12"))
        for letter, arr, pre in (("E", strain, "e"), ("S", stress, "s")):
            if letter not in fields:
                continue
            for k, nm in enumerate(names):
                rec = np.transpose(arr[:, :, k, :], (2, 1, 0))  # record e, i fastest
                np.ascontiguousarray(rec, dtype="<f4").tofile(os.path.join(path, "%s%s_%s_sem2d.dat" % (pre, nm, tag)))


def _write_divcurl(path, tag, v, grid, fields):
    """div v = dvx/dx + dvz/dz and curl v = dvx/dz - dvz/dx at the element
    GLL points of the Cartesian mesher's rectangular elements (dxi/dz =
    deta/dx = 0), records as for the strain."""
    ib = grid.ibool() - 1  # (ngll, ngll, nelem)
    xz = grid.coord()
    _, _, H = grid.gll()  # H[k, i] = h'_k(x_i)
    N = ib.shape[0]
    vx, vz = v[:, 0][ib], v[:, 1][ib]
    dxi_dx = 2.0 / (xz[0][ib[N - 1, 0, :]] - xz[0][ib[0, 0, :]])
    deta_dz = 2.0 / (xz[1][ib[0, N - 1, :]] - xz[1][ib[0, 0, :]])
    dxi = lambda u: np.einsum("ki,kje->ije", H, u)   # Ht . u
    deta = lambda u: np.einsum("ike,kj->ije", u, H)  # u . H
    out = {"d": ("div", dxi(vx) * dxi_dx + deta(vz) * deta_dz),
           "c": ("curl", deta(vx) * deta_dz - dxi(vz) * dxi_dx)}
    for letter in "dc":
        if letter in fields:
            name, arr = out[letter]
            rec = np.transpose(arr, (2, 1, 0))  # record e, i fastest
            np.ascontiguousarray(rec, dtype="<f4").tofile(os.path.join(path, "%s_%s_sem2d.dat" % (name, tag)))


def write_run(path, solver, problem):
    """Every output file of a run the reference would have written for its
    deck: the grid files, seismograms, and for a fault its records (and the
    potency when the handle keeps it).  `solver` a Solver (or an oracle run with the same
    getters), `problem` the Problem it was created from."""
    d = solver.desc
    write_grid(path, problem.grid)
    if d.nrec:
        write_seismograms(path, solver.seismograms(), d.rec_isamp * d.dt, problem.rec_coord())
    if d.nflt:
        tag = problem.deck.fault.tags[0] if problem.deck.fault is not None else 5
        xz = problem.fault_coord()
        series = solver.fault_series()
        if xz.shape[1] != series.shape[0]:
            xz = xz[:, (d.flt_oix1 - 1):d.flt_oixn:d.flt_oixd]
        write_fault(path, tag, series, d.flt_oitd * d.dt, xz)
        if getattr(d, "flt_potency", 0):
            write_potency(path, tag, solver.fault_potency(), d.ndof)
