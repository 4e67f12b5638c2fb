"""Par.inp-shaped problem description.

Each class mirrors one NAMELIST block of the reference input file
(doc/doc.txt; the *_read routines cited below) for the Cartesian solver
path.  ``ParDeck.to_c()`` packs the values into the ``sem2d_deck`` C struct
of include/sem2d_host.h and keeps the numpy arrays it points to alive.
"""
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple, Union

import ctypes as C
import numpy as np

from . import abi

ArrayLike = Union[float, np.ndarray]


def _dptr(a):
    return a.ctypes.data_as(abi.P_double) if a is not None else abi.P_double()


@dataclass
class Material:
    """&MATERIAL tag + &MAT_ELASTIC (mat_elastic.f90:69-189) [+ &MAT_KV]."""
    tag: int = 1
    rho: float = 0.0
    cp: float = 0.0
    cs: float = 0.0
    c11: float = 0.0
    c13: float = 0.0
    c33: float = 0.0
    c55: float = 0.0
    c66: float = 0.0
    aniso: bool = False
    hetero: bool = False      # values taken from ParDeck.hetero arrays
    kv_eta: Optional[float] = None
    kv_etaxdt: bool = True


@dataclass
class TimeWeakening:
    """&BC_DYNFLT_TWF (bc_dynflt_twf.f90:52-100), reference defaults."""
    kind: int = 1
    mus: float = 0.6
    mud: float = 0.5
    mu0: float = 0.6
    X: float = 0.0
    Z: float = 0.0
    V: float = 1e3
    L: float = 1.0
    T: float = float(np.finfo(np.float64).max)
    Dc: float = float(np.finfo(np.float64).max)


@dataclass
class Fault:
    """&BC_DEF kind='DYNFLT' + &BC_DYNFLT/_SWF/_RSF/_TWF/_NOR (bc_dynflt.f90:100-178).

    ``friction`` is 'SWF', 'RSF' or 'TWF'; ``twf`` adds a time-weakening law,
    superimposed on SWF/RSF (friction='SWF','TWF' in Par.inp) or alone.
    """
    tags: Tuple[int, int] = (5, 6)
    friction: str = "SWF"
    twf: Optional[TimeWeakening] = None
    swf_kind: int = 1
    healing: bool = False
    rsf_kind: int = 1
    normal_kind: int = 1
    normal_T: float = 1.0
    normal_L: float = 1.0
    normal_V: float = 1.0
    opening: bool = True
    ot1: float = 0.0
    otd: float = 0.0
    oxi: Tuple[int, int, int] = (1, 0, 1)
    # record the potency of displacement and velocity every step
    potency: bool = False
    # name (abi.FP_NAMES) -> scalar, or an array over the fault nodes
    values: Dict[str, ArrayLike] = field(default_factory=dict)


@dataclass
class Time:
    """&TIME (+ &TIME_NEWMARK or &TIME_HHTA) (time.f90:122-315)."""
    kind: str = "leapfrog"
    dt: float = 0.0
    courant: float = 0.5
    total_time: float = 0.0
    nsteps: int = 0
    beta: float = 0.0
    gamma: float = 0.5
    alpha: float = 0.5   # &TIME_HHTA (kind 'hht-alpha')
    rho: float = 0.5


@dataclass
class Stf:
    """A source time function, &SRC_DEF stf= + its &STF_* block
    (stf_gen.f90:45-97): kind 'RICKER', 'GAUSSIAN' (f0, onset, ampli),
    'BRUNE' (f0 = the corner frequency fc, ampli), 'HARMONIC' (f0, ampli),
    'USER' (onset, ampli, par1, par2) or 'TAB' (tab = (t, v) rows of the
    reference's stf.tab file).  Values as written in the input."""
    kind: str = "RICKER"
    f0: float = 0.0
    onset: float = 0.0
    ampli: float = 1.0
    par1: float = 0.0
    par2: float = 0.0
    tab: Optional[Tuple[Sequence[float], Sequence[float]]] = None

    def to_c(self, keep):
        s = abi.Stf()
        kind = self.kind.upper()
        if kind not in abi.STF_KINDS:
            raise ValueError("source time function %s is not on the GPU path" % self.kind)
        s.kind = abi.STF_KINDS[kind]
        s.f0, s.onset, s.ampli = float(self.f0), float(self.onset), float(self.ampli)
        s.par1, s.par2 = float(self.par1), float(self.par2)
        if s.kind == abi.STF_TAB:
            if self.tab is None:
                raise ValueError("TAB time function without rows")
            t = np.ascontiguousarray(np.asarray(self.tab[0], dtype=np.float64))
            v = np.ascontiguousarray(np.asarray(self.tab[1], dtype=np.float64))
            if t.shape != v.shape or t.ndim != 1:
                raise ValueError("TAB time function: t and v must be 1-D of one length")
            keep += [t, v]
            s.ntab = t.size
            s.tab_t, s.tab_v = _dptr(t), _dptr(v)
        return s


@dataclass
class Sources:
    """&SRC_DEF + &STF_* + &SRC_FORCE / &SRC_MOMENT / &SRC_WAVE.

    ``stf`` None is the Ricker of f0, onset, ampli (&STF_RICKER).  With
    mechanism 'WAVE' the first source is an incident plane wave
    (src_wave.f90): wave_angle in degrees counterclockwise from z up to the
    wave vector, wave_phase 'P' or 'S' (ignored in SH)."""
    coords: Sequence[Sequence[float]] = ((0.0, 0.0),)
    f0: float = 1.0
    onset: float = 1.0
    ampli: float = 1.0
    angle: float = 0.0
    tdelay: Optional[Sequence[float]] = None
    relamp: Optional[Sequence[float]] = None
    # mechanism (src_moment.f90): FORCE (angle), EXPLOSION, DOUBLE_COUPLE
    # (dip, degrees) or MOMENT (M = Mxx, Mxz, Mzx, Mzz; SH: Myx, Myz)
    mechanism: str = "FORCE"
    dip: float = 90.0
    M: Tuple[float, float, float, float] = (0.0, 0.0, 0.0, 0.0)
    stf: Optional[Stf] = None
    wave_angle: float = 0.0
    wave_phase: str = "S"


@dataclass
class Layer:
    """One layer of &MESH_DEF method='LAYERED' (&MESH_LAYER nz, ztop or
    ztopH, tag; mesh_layers.f90:212-300): its element rows, material tag
    and top boundary, a height or a distribution of x (a Dist evaluated at
    z = 0).  `quadratic`: Q9 elements (a top other than flat or LINEAR)."""
    nz: int = 1
    tag: int = 1
    ztop: Union[float, object] = 0.0
    quadratic: bool = False


@dataclass
class Receivers:
    """&REC_LINE (receivers.f90:62-163)."""
    number: int = 0
    first: Tuple[float, float] = (0.0, 0.0)
    last: Tuple[float, float] = (0.0, 0.0)
    coords: Optional[np.ndarray] = None
    atnode: bool = True
    isamp: int = 1
    field: str = "V"


@dataclass
class ParDeck:
    """The blocks of one Par.inp for the Cartesian solver path."""
    ngll: int = 5
    ndof: int = 2
    fmax: float = 1.0
    xlim: Tuple[float, float] = (0.0, 1.0)
    zlim: Tuple[float, float] = (0.0, 1.0)
    nelem: Tuple[int, int] = (1, 1)
    ezflt: int = 0
    fztag: int = 0
    fznz: int = 1
    domains: List[Tuple[int, Tuple[int, int], Tuple[int, int]]] = field(default_factory=list)
    materials: List[Material] = field(default_factory=list)
    absorbing: List[int] = field(default_factory=list)   # tags with kind='ABSORB'
    stacey: List[int] = field(default_factory=list)      # of those, the tags with &BC_ABSORB stacey=T
    # &BC_DEF kind='DIRNEU' + &BC_DIRNEU h, v: (tag, h, v, before_fault), h and
    # v 'N' or 'D'; before_fault when the block precedes the fault's in &BC_DEF
    dirneu: List[Tuple[int, str, str, bool]] = field(default_factory=list)
    # &BC_DIRNEU hstf, vstf: tag -> (Stf or None, Stf or None), the time
    # functions of the horizontal and vertical tractions of a Neumann side
    dirneu_stf: Dict[int, Tuple[Optional[Stf], Optional[Stf]]] = field(default_factory=dict)
    # absorbing tags with &BC_ABSORB let_wave=F
    no_wave: List[int] = field(default_factory=list)
    # &BC_DEF kind='PERIOD' tags=(master, slave)
    periodic: Optional[Tuple[int, int]] = None
    fault: Optional[Fault] = None
    fault_first: bool = False  # &BC_DEF order: DYNFLT block before the ABSORB blocks
    time: Time = field(default_factory=Time)
    sources: Optional[Sources] = None
    receivers: Optional[Receivers] = None
    precision: int = abi.PRECISION_FP64
    kd2_form: int = -1
    width: float = 0.0   # W of &GENERAL; 0 = 2D (the reference's huge)
    # per element GLL point arrays (ngll,ngll,nelem) for hetero materials
    hetero: Dict[str, np.ndarray] = field(default_factory=dict)
    # &MESH_DEF method 'CARTESIAN' or 'LAYERED' (&MESH_LAYERED xlim, zmin,
    # nx = nelem[0], ezflt, fztag, fznz; `layers` from the bottom up)
    mesh: str = "CARTESIAN"
    zmin: float = 0.0
    layers: List[Layer] = field(default_factory=list)

    def layer_abscissae(self):
        """x of the control-node columns of a layered mesh (mesh_layers.f90:
        357-361): nxp = nx+1 with Q4 elements, 2 nx+1 with Q9."""
        d = 2 if any(layer.quadratic for layer in self.layers) else 1
        nxp = d * int(self.nelem[0]) + 1
        x0, x1 = float(self.xlim[0]), float(self.xlim[1])
        return np.array([x0 + (x1 - x0) / float(nxp - 1) * float(i) for i in range(nxp)])

    def to_c(self):
        """Return (abi.Deck, keepalive) for the C builders."""
        keep = []
        d = abi.Deck()
        d.ngll, d.ndof, d.fmax = self.ngll, self.ndof, float(self.fmax)
        d.xlim[:] = [float(v) for v in self.xlim]
        d.zlim[:] = [float(v) for v in self.zlim]
        d.nelem[:] = [int(v) for v in self.nelem]
        d.ezflt, d.fztag, d.fznz = self.ezflt, self.fztag, self.fznz
        if len(self.domains) > abi.MAX_DOMAINS or len(self.materials) > abi.MAX_MATS:
            raise ValueError("too many domains or materials")
        d.ndomains = len(self.domains)
        for k, (tag, ex, ez) in enumerate(self.domains):
            d.domains[k].tag = tag
            d.domains[k].ex[:] = list(ex)
            d.domains[k].ez[:] = list(ez)
        d.nmats = len(self.materials)
        for k, m in enumerate(self.materials):
            cm = d.mats[k]
            cm.tag, cm.aniso, cm.hetero = m.tag, int(m.aniso), int(m.hetero)
            cm.rho, cm.cp, cm.cs = m.rho, m.cp, m.cs
            cm.c11, cm.c13, cm.c33, cm.c55, cm.c66 = m.c11, m.c13, m.c33, m.c55, m.c66
            cm.kv = int(m.kv_eta is not None)
            cm.kv_eta = float(m.kv_eta or 0.0)
            cm.kv_etaxdt = int(m.kv_etaxdt)
        for name in ("rho", "cp", "cs", "c11", "c13", "c33", "c55", "c66", "kveta"):
            arr = self.hetero.get(name)
            if arr is not None:
                arr = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).ravel(order="F"))
                keep.append(arr)
            setattr(d, "h_" + name, _dptr(arr))
        for t in self.stacey:
            if t not in self.absorbing:
                raise ValueError("stacey tag %d is not an absorbing boundary" % t)
        pre, post = [], []
        for t, h, v, before in self.dirneu:
            if h not in "ND" or v not in "ND" or len(h) != 1 or len(v) != 1:
                raise ValueError("BC_DIRNEU h and v must be 'N' or 'D'")
            (pre if before else post).append((abi.BC_DIRNEU, (t, (h == "D") | ((v == "D") << 1))))
        absorb = [(abi.BC_ABSORB, (t, 0)) for t in self.absorbing]
        if self.periodic is not None:
            absorb = [(abi.BC_PERIOD, tuple(self.periodic))] + absorb
        if self.fault is None:
            bcs = absorb + pre + post
        elif self.fault_first:
            bcs = pre + [(abi.BC_DYNFLT, self.fault.tags)] + absorb + post
        else:
            bcs = absorb + pre + [(abi.BC_DYNFLT, self.fault.tags)] + post
        if len(bcs) > abi.MAX_BCS:
            raise ValueError("too many boundary conditions")
        d.nbcs = len(bcs)
        for t in self.dirneu_stf:
            if t not in [q[0] for q in self.dirneu]:
                raise ValueError("traction time functions for tag %d, which is not a DIRNEU side" % t)
        for k, (kind, tags) in enumerate(bcs):
            d.bcs[k].kind = kind
            if kind == abi.BC_DIRNEU:
                d.bcs[k].tag[:] = [int(tags[0]), 0]
                d.bcs[k].dirichlet = int(tags[1])
                hs, vs = self.dirneu_stf.get(int(tags[0]), (None, None))
                if hs is not None:
                    d.bcs[k].hstf = hs.to_c(keep)
                if vs is not None:
                    d.bcs[k].vstf = vs.to_c(keep)
                continue
            d.bcs[k].tag[:] = [int(tags[0]), int(tags[1])]
            d.bcs[k].stacey = int(kind == abi.BC_ABSORB and tags[0] in self.stacey)
            d.bcs[k].no_wave = int(kind == abi.BC_ABSORB and tags[0] in self.no_wave)
        f = self.fault
        for i, name in enumerate(abi.FP_NAMES):
            d.flt_value[i] = abi.FP_DEFAULTS[name]
            d.flt_array[i] = abi.P_double()
        if f is not None:
            d.flt_friction = {"RSF": abi.FRICTION_RSF, "TWF": abi.FRICTION_TWF}.get(
                f.friction.upper(), abi.FRICTION_SWF)
            tw = f.twf
            if tw is None and d.flt_friction == abi.FRICTION_TWF:
                tw = TimeWeakening()
            if tw is not None:
                d.twf_kind = tw.kind
                d.twf_mus, d.twf_mud, d.twf_mu0 = tw.mus, tw.mud, tw.mu0
                d.twf_X, d.twf_Z, d.twf_V, d.twf_L = tw.X, tw.Z, tw.V, tw.L
                d.twf_T, d.twf_Dc = tw.T, tw.Dc
            d.swf_kind, d.swf_healing, d.rsf_kind = f.swf_kind, int(f.healing), f.rsf_kind
            d.normal_kind = f.normal_kind
            d.normal_T, d.normal_L, d.normal_V = f.normal_T, f.normal_L, f.normal_V
            d.flt_opening = int(f.opening)
            d.flt_potency = int(f.potency)
            d.flt_ot1, d.flt_otd = f.ot1, f.otd
            d.flt_oxi[:] = list(f.oxi)
            for name, val in f.values.items():
                i = abi.FP_INDEX[name]
                if np.isscalar(val):
                    d.flt_value[i] = float(val)
                else:
                    arr = np.ascontiguousarray(np.asarray(val, dtype=np.float64))
                    keep.append(arr)
                    d.flt_array[i] = _dptr(arr)
        t = self.time
        kinds = {"leapfrog": abi.TIME_LEAPFROG, "newmark": abi.TIME_NEWMARK, "hht-alpha": abi.TIME_HHT}
        if t.kind.lower() not in kinds:
            raise ValueError("time scheme %s is not on the GPU path" % t.kind)
        d.time_kind = kinds[t.kind.lower()]
        d.hht_alpha, d.hht_rho = t.alpha, t.rho
        d.dt, d.courant, d.total_time, d.nsteps = t.dt, t.courant, t.total_time, t.nsteps
        d.beta, d.gamma = t.beta, t.gamma
        s = self.sources
        if s is not None:
            xy = np.ascontiguousarray(np.asarray(s.coords, dtype=np.float64).reshape(-1, 2))
            keep.append(xy)
            d.nsrc = xy.shape[0]
            d.src_coord = _dptr(xy)
            for attr, val in (("src_tdelay", s.tdelay), ("src_ampli", s.relamp)):
                if val is not None:
                    arr = np.ascontiguousarray(np.asarray(val, dtype=np.float64))
                    keep.append(arr)
                    setattr(d, attr, _dptr(arr))
            d.ricker_f0, d.ricker_onset, d.ricker_ampli = s.f0, s.onset, s.ampli
            d.force_angle = s.angle
            mechs = {"FORCE": 0, "EXPLOSION": 1, "DOUBLE_COUPLE": 2, "MOMENT": 3, "WAVE": 4}
            if s.mechanism.upper() not in mechs:
                raise ValueError("source mechanism %s is not on the GPU path" % s.mechanism)
            d.src_mech = mechs[s.mechanism.upper()]
            d.src_M[:] = [float(v) for v in s.M]
            d.src_dip = s.dip
            if s.stf is not None:
                d.stf = s.stf.to_c(keep)
            d.wave_angle = float(s.wave_angle)
            phases = {"P": abi.WAVE_P, "S": abi.WAVE_S}
            if s.wave_phase.upper() not in phases:
                raise ValueError("WAVE_read: phase must be S or P")
            d.wave_phase = phases[s.wave_phase.upper()]
        r = self.receivers
        if r is not None:
            if r.coords is not None:
                rc = np.ascontiguousarray(np.asarray(r.coords, dtype=np.float64).reshape(-1, 2))
                keep.append(rc)
                d.rec_number = rc.shape[0]
                d.rec_coord = _dptr(rc)
            else:
                d.rec_number = r.number
            d.rec_first[:] = list(r.first)
            d.rec_last[:] = list(r.last)
            d.rec_atnode, d.rec_isamp = int(r.atnode), r.isamp
            d.rec_field = r.field.encode()[:1]
        d.precision, d.kd2_form = self.precision, self.kd2_form
        d.width = float(self.width)
        if self.mesh.upper() == "LAYERED":
            if not self.layers or len(self.layers) > abi.MAX_LAYERS:
                raise ValueError("MESH_LAYERS_read: nlayer or file must be set")
            d.mesh_method, d.zmin, d.nlayer = 1, float(self.zmin), len(self.layers)
            x = self.layer_abscissae()
            for k, layer in enumerate(self.layers):
                d.layer_nz[k], d.layer_tag[k] = int(layer.nz), int(layer.tag)
                d.layer_ngnod[k] = 9 if layer.quadratic else 4
                if callable(layer.ztop):
                    top = np.asarray(layer.ztop(x, np.zeros_like(x)), dtype=np.float64)
                else:
                    top = np.full(x.shape, float(layer.ztop))
                top = np.ascontiguousarray(top)
                keep.append(top)
                d.layer_top[k] = _dptr(top)
        elif self.mesh.upper() != "CARTESIAN":
            raise ValueError("only the CARTESIAN and LAYERED meshers are on the GPU path")
        return d, keep
