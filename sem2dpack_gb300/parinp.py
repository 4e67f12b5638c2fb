"""Par.inp front end: the reference's input file (Fortran NAMELIST blocks,
doc/doc.txt) read into a :class:`~sem2dpack_gb300.deck.ParDeck` for the
Cartesian solver path.

``read_namelists(text)`` returns the blocks in file order, each a
(name, {key: value}) pair; values are Python scalars or lists (Fortran
``d`` exponents, ``T``/``F`` logicals, quoted strings, ``r*value`` repeats).
As Fortran's namelist read does, a block ends at the first ``/``; text
between blocks (``#`` comments, anything after the ``/``) is ignored.

``deck_from_parinp(text)`` maps the blocks the GPU path supports:

  &GENERAL      ngll, ndof, fmax, W (2.5D width)            (input.f90 / init)
  &MESH_DEF     method='CARTESIAN' + &MESH_CART xlim, zlim, nelem, ezflt,
                FaultX... (mesh_cartesian.f90:86-200) + &MESH_CART_DOMAIN
  &MATERIAL     tag, kind 'ELAST' [+ 'KV'] + &MAT_ELASTIC rho, cp, cs or
                c11, c13, c33, c55, c66 (mat_elastic.f90:69-189),
                &MAT_KV eta, ETAxDT (mat_kelvin_voigt.f90)
  &BC_DEF       tag, kind 'ABSORB' + &BC_ABSORB stacey (bc_abso.f90),
                kind 'DIRNEU' + &BC_DIRNEU h, v (bc_dirneu.f90:50-112),
                kind 'PERIOD' tags (bc_periodic.f90),
                kind 'DYNFLT' + &BC_DYNFLT / _SWF / _RSF / _TWF / _NOR with
                scalar values (bc_dynflt*.f90)
  &TIME         kind, Dt, Courant, TotalTime, NbSteps + &TIME_NEWMARK or &TIME_HHTA alpha, rho
                beta, gamma (time.f90:122-315)
  &SRC_DEF      stf 'RICKER', 'GAUSSIAN', 'BRUNE', 'HARMONIC', 'TAB' or 'USER'
                + its &STF_* block (stf_*.f90); mechanism 'FORCE' + &SRC_FORCE
                angle, 'EXPLOSION', 'DOUBLE_COUPLE', 'MOMENT' (src_moment.f90) or
                'WAVE' + &SRC_WAVE angle, phase (src_wave.f90); coord or file
  &BC_ABSORB    stacey, let_wave; &BC_DIRNEU hstf, vstf + their &STF_* blocks
  &REC_LINE     number, first, last or file, field, isamp, AtNode (receivers.f90)

and names the blocks it skips in ``deck.skipped``: plots, snapshots,
energies, and the option blocks the reference would not read for this deck
(as it does, a &SRC_WAVE next to a mechanism='FORCE' source, or a
&MESH_EMC2 under method='CARTESIAN', is ignored).  A selecting block that
asks for something off the GPU path (another mesher, material kind,
boundary kind, source mechanism, time function or time scheme, a SPLINE or
HETE1 distribution) raises ValueError.

Material and fault values given as distributions (rhoH, cpH, csH, etaH,
TtH, TnH, MuSH, DcH, aH, ... followed by &DIST_* blocks) are evaluated on
the host (sem2dpack_gb300.distributions) at the fault nodes and at the
element GLL points once the grid is built.
"""
import os
import re

import numpy as np

from .deck import Fault, Material, ParDeck, Receivers, Sources, TimeWeakening, Time
from .distributions import Dist

__all__ = ["read_namelists", "read_blocks", "deck_from_parinp", "load_parinp"]

TIME_KINDS = ("leapfrog", "newmark", "hht-alpha")

_TOKEN = re.compile(r"""'[^']*'|"[^"]*"|[&/=,]|[^\s&/=,'"]+""")


def _strip_comments(text):
    out = []
    for line in text.splitlines():
        s, q = [], None
        for ch in line:
            if q:
                s.append(ch)
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                s.append(ch)
            elif ch in "#!":
                break
            else:
                s.append(ch)
        out.append("".join(s))
    return "\n".join(out)


def _value(tok):
    if tok[0] in "'\"":
        return tok[1:-1]
    low = tok.lower()
    if low in ("t", ".true.", "true"):
        return True
    if low in ("f", ".false.", "false"):
        return False
    try:
        return int(tok)
    except ValueError:
        pass
    try:
        return float(low.replace("d", "e"))
    except ValueError:
        return tok


def read_namelists(text):
    """[(NAME, {key: value or [values]})] in file order."""
    return [(name, items) for name, items, _ in read_blocks(text)]


def read_blocks(text):
    """[(NAME, items, data)] in file order; data are the free-format values
    between the block's closing '/' and the next '&' (the tables that
    follow &DIST_PWCONR, &DIST_ORDER0 or &DIST_LINEAR)."""
    toks = _TOKEN.findall(_strip_comments(text))
    blocks, k = [], 0
    while k < len(toks):
        if toks[k] != "&" or k + 1 >= len(toks):
            if blocks and toks[k] not in ",/":
                blocks[-1][2].append(_value(toks[k]))
            k += 1
            continue
        name, k = toks[k + 1].upper(), k + 2
        items, key, vals = {}, None, []
        while k < len(toks) and toks[k] != "/":
            t = toks[k]
            if k + 1 < len(toks) and toks[k + 1] == "=" and t not in ",=&":
                if key is not None:
                    items[key] = vals[0] if len(vals) == 1 else vals
                key, vals, k = t.lower(), [], k + 2
                continue
            if t not in ",":
                m = re.fullmatch(r"(\d+)\*(.+)", t)
                if m and t[0] not in "'\"":
                    vals.extend([_value(m.group(2))] * int(m.group(1)))
                else:
                    vals.append(_value(t))
            k += 1
        if key is not None:
            items[key] = vals[0] if len(vals) == 1 else vals
        blocks.append((name, items, []))
        k += 1
    return blocks


def _pair(v):
    return (float(v[0]), float(v[1]))


# parameters that may be given as distributions (name + 'H'), in the order
# the reference's read routines consume the &DIST_* blocks that follow
_FAULT_DIST = (("cohesion", "cohesion"), ("tn", "Tn"), ("tt", "Tt"), ("sxx", "Sxx"), ("sxy", "Sxy"),
               ("sxz", "Sxz"), ("syz", "Syz"), ("szz", "Szz"), ("v", "V"))   # bc_dynflt.f90:162-170
_SWF_DIST = (("dc", "swf_dc"), ("mus", "swf_mus"), ("mud", "swf_mud"), ("alpha", "swf_alpha"),
             ("p", "swf_p"))                                                  # bc_dynflt_swf.f90:99-103
_RSF_DIST = (("dc", "rsf_dc"), ("mus", "rsf_mus"), ("a", "rsf_a"), ("b", "rsf_b"), ("vstar", "rsf_vstar"),
             ("theta", "rsf_theta"), ("vc", "rsf_vc"))                         # bc_dynflt_rsf.f90:112-118


def deck_from_parinp(text, precision=None, base=None):
    """ParDeck for the Par.inp text (see the module docstring).  `base` is
    the folder that `file=` names in &DIST_* blocks are relative to."""
    blocks3 = read_blocks(text)
    blocks = [(n, i) for n, i, _ in blocks3]
    consumed = set()
    fault_dists, mat_dists = {}, {}

    def take_dists(j, it, keys):
        """{name: Dist} for the keys of block j given as distributions: each
        reads the next &DIST_<kind> block after the ones already read, as
        the reference's namelist reads search forward (distribution_cd.f90
        DIST_CD_Read)."""
        out, pos = {}, j + 1
        for key, name in keys:
            v = it.get(key + "h")
            if v is None or str(v).strip() == "":
                continue
            want = "DIST_" + str(v).strip().upper()
            q = pos
            while q < len(blocks3) and blocks3[q][0] != want:
                q += 1
            if q >= len(blocks3):
                raise ValueError("&%s %sH='%s': no &%s block follows" % (blocks3[j][0], key, v, want))
            consumed.add(q)
            out[name] = Dist(want[5:], blocks3[q][1], blocks3[q][2], base)
            pos = q + 1
        return out

    def take_stf(j, sname):
        """Stf of the first &STF_<sname> block after block j (STF_read,
        stf_gen.f90:45-97: the namelist read searches forward from the
        block that names the function), and its index."""
        sname = str(sname).strip().upper()
        if sname not in ("RICKER", "GAUSSIAN", "BRUNE", "HARMONIC", "TAB", "USER"):
            raise ValueError("source time function %s is not on the GPU path" % sname)
        q = j + 1
        while q < len(blocks) and blocks[q][0] != "STF_" + sname:
            q += 1
        if q >= len(blocks):
            if sname == "TAB":  # &STF_TAB is optional: file = 'stf.tab'
                return _stf_values(sname, {}, base), j
            raise ValueError("%s: input block STF_%s not found" % (sname, sname))
        consumed.add(q)
        return _stf_values(sname, blocks[q][1], base), q

    kw = {}
    if precision is not None:
        kw["precision"] = precision
    deck = ParDeck(**kw)
    deck.skipped = []
    mats, fault, cur_bc, absorbing = [], None, None, []
    time = Time()
    src, rec = None, None
    domains = []
    k = 0
    while k < len(blocks):
        name, it = blocks[k]
        nxt = blocks[k + 1] if k + 1 < len(blocks) else ("", {})
        if k in consumed:
            k += 1
            continue
        if name == "GENERAL":
            deck.ngll = int(it.get("ngll", deck.ngll))
            deck.ndof = int(it.get("ndof", deck.ndof))
            deck.fmax = float(it.get("fmax", deck.fmax))
            if float(it.get("w", 0.0) or 0.0) > 0.0:
                deck.width = float(it["w"])
        elif name == "MESH_DEF":
            method = str(it.get("method", "CARTESIAN")).upper()
            if method not in ("CARTESIAN", "LAYERED"):
                raise ValueError("only &MESH_DEF method='CARTESIAN' or 'LAYERED' is on the GPU path")
            deck.mesh = method
        elif name == "MESH_LAYERED" and deck.mesh == "LAYERED":
            # MESH_LAYERS_read (mesh_layers.f90:30-88): &MESH_LAYERED, then
            # nlayer &MESH_LAYER blocks (each followed by its &DIST_* block
            # when ztopH is set) or a file of "ztop nz tag" lines, listed from
            # the top down; default tags 1 (top) to nlayer (bottom)
            xl = it.get("xlim")
            if xl is None or "zmin" not in it:
                raise ValueError("MESH_LAYERS_read: you must set xlim and zmin")
            deck.xlim = _pair(xl)
            deck.zmin = float(it["zmin"])
            nx = int(it.get("nx", 1))
            deck.ezflt = int(it.get("ezflt", 0))
            deck.fztag = int(it.get("fztag", 0)) if deck.ezflt != 0 else 0
            deck.fznz = int(it.get("fznz", 1))
            f = str(it.get("file", "")).strip()
            from .deck import Layer
            top_down = []
            if f:
                for row in np.loadtxt(os.path.join(base or ".", f), ndmin=2):
                    top_down.append(Layer(nz=int(row[1]), tag=int(row[2]), ztop=float(row[0])))
            else:
                nl = int(it.get("nlayer", 0))
                if nl <= 0:
                    raise ValueError("MESH_LAYERS_read: nlayer or file must be set")
                q = k + 1
                for li in range(nl):
                    while q < len(blocks) and blocks[q][0] != "MESH_LAYER":
                        q += 1
                    if q >= len(blocks):
                        raise ValueError("MESH_LAYERS_read: %d &MESH_LAYER blocks expected" % nl)
                    consumed.add(q)
                    b = blocks[q][1]
                    layer = Layer(nz=int(b.get("nz", 0)), tag=int(b.get("tag", li + 1)))
                    zh = str(b.get("ztoph", "")).strip().upper()
                    if zh in ("QSPLINE", "CSPLINE"):
                        raise ValueError("&MESH_LAYER ztopH='%s' is not supported by the front end" % zh)
                    if zh:
                        dist = take_dists(q, {"ztoph": zh}, [("ztop", "ztop")])["ztop"]
                        layer.ztop, layer.quadratic = dist, zh != "LINEAR"
                    elif "ztop" in b:
                        layer.ztop = float(b["ztop"])
                    else:
                        raise ValueError("MESH_LAYERS_read: ztop or ztopH must be set")
                    top_down.append(layer)
                    q += 1
            if any(layer.nz <= 0 for layer in top_down):
                raise ValueError("MESH_LAYERS_read: nz null, negative or missing")
            deck.layers = top_down[::-1]
            deck.nelem = (nx, sum(layer.nz for layer in top_down))
        elif name == "MESH_CART":
            deck.xlim = _pair(it["xlim"])
            deck.zlim = _pair(it["zlim"])
            ne = it["nelem"]
            deck.nelem = (int(ne[0]), int(ne[1]))
            deck.ezflt = int(it.get("ezflt", 0))
            deck.fztag = int(it.get("fztag", 0))
            deck.fznz = int(it.get("fznz", 1))
        elif name == "MESH_CART_DOMAIN":
            ex, ez = it["ex"], it["ez"]
            domains.append((int(it["tag"]), (int(ex[0]), int(ex[1])), (int(ez[0]), int(ez[1]))))
        elif name == "MATERIAL":
            kinds = it.get("kind", "ELAST")
            kinds = [kinds] if isinstance(kinds, str) else list(kinds)
            m = Material(tag=int(it.get("tag", 1)))
            kinds = [s.upper() for s in kinds]
            if any(s not in ("ELAST", "KV") for s in kinds):
                raise ValueError("material kind %s is not on the GPU path" % kinds)
            # MAT_read (mat_gen.f90:134-195): each kind's block is the first
            # of its name after this &MATERIAL block (namelist reads search
            # forward), so materials may share one &MAT_ELASTIC
            md = {}
            for kname in kinds:
                want = "MAT_ELASTIC" if kname == "ELAST" else "MAT_KV"
                j = k + 1
                while j < len(blocks) and blocks[j][0] != want:
                    j += 1
                if j >= len(blocks):
                    if kname == "ELAST":
                        raise ValueError("&MATERIAL tag=%d: no &MAT_ELASTIC block follows" % m.tag)
                    continue
                bn, b = blocks[j]
                consumed.add(j)
                if bn == "MAT_ELASTIC":
                    # MAT_ELAST_read (mat_elastic.f90:102-135): rho, then cp, cs or the c_ij
                    aniso = any(c in b or c + "h" in b for c in ("c11", "c55"))
                    props = ("rho", "c11", "c13", "c33", "c55", "c66") if aniso else ("rho", "cp", "cs")
                    md.update(take_dists(j, b, [(c, c) for c in props]))
                    m.aniso = aniso
                    for c in props:
                        setattr(m, c, float(b.get(c, 0.0)))
                else:
                    md.update(take_dists(j, b, [("eta", "kveta")]))
                    m.kv_eta = float(b.get("eta", 0.0))
                    m.kv_etaxdt = bool(b.get("etaxdt", True))
            if md:
                mat_dists[m.tag] = md
            mats.append(m)
        elif name == "BC_DEF":
            kind = str(it.get("kind", "")).upper()
            tags = it.get("tags", it.get("tag"))
            tags = [tags] if not isinstance(tags, list) else tags
            cur_bc = kind
            if kind == "ABSORB":
                absorbing.extend(int(t) for t in tags)
                if nxt[0] == "BC_ABSORB" and nxt[1].get("stacey", False):
                    deck.stacey.extend(int(t) for t in tags)
                if nxt[0] == "BC_ABSORB" and not nxt[1].get("let_wave", True):
                    deck.no_wave.extend(int(t) for t in tags)
            elif kind == "DYNFLT":
                fault = fault or Fault()
                # a single tag is a one-sided fault: tags = (tag, 0) (bc_gen.f90:126-133)
                fault.tags = (int(tags[0]), int(tags[1]) if len(tags) > 1 else 0)
                deck.fault_first = not absorbing
            elif kind == "PERIOD":
                if len(tags) != 2:
                    raise ValueError("&BC_DEF kind='PERIOD' needs two tags")
                deck.periodic = (int(tags[0]), int(tags[1]))
            elif kind == "DIRNEU":
                b = nxt[1] if nxt[0] == "BC_DIRNEU" else {}
                extra = set(b) - {"h", "v", "hstf", "vstf"}
                if extra:
                    raise ValueError("&BC_DIRNEU %s is not on the GPU path" % ", ".join(sorted(extra)))
                h, v = str(b.get("h", "N")).upper(), str(b.get("v", "N")).upper()
                deck.dirneu.extend((int(t), h, v, fault is None) for t in tags)
                # bc_DIRNEU_read (bc_dirneu.f90:50-112): the time function of a
                # Neumann component reads the next &STF_* block, h then v; a
                # Dirichlet component's name is reset to 'none'
                pos, stfs = k + 1, [None, None]
                for c, (key, bcc) in enumerate((("hstf", h), ("vstf", v))):
                    name_c = str(b.get(key, "none")).strip()
                    if bcc == "D" or name_c.lower() == "none":
                        continue
                    stfs[c], pos = take_stf(pos, name_c)
                if stfs[0] is not None or stfs[1] is not None:
                    for t in tags:
                        deck.dirneu_stf[int(t)] = (stfs[0], stfs[1])
            else:
                raise ValueError("boundary kind %s is not on the GPU path" % kind)
        elif name in ("BC_ABSORB", "BC_DIRNEU"):
            pass
        elif name == "BC_DYNFLT":
            fault = fault or Fault()
            fr = it.get("friction", "SWF")
            fr = [fr] if isinstance(fr, str) else list(fr)
            fr = [s.upper() for s in fr]
            fault.friction = fr[0]
            if "TWF" in fr and fr[0] != "TWF":
                fault.twf = fault.twf or TimeWeakening()
            fault.opening = bool(it.get("opening", True))
            for key, fname in _FAULT_DIST:
                if key in it:
                    fault.values[fname] = float(it[key])
            fault_dists.update(take_dists(k, it, _FAULT_DIST))
            if "ot1" in it:
                fault.ot1 = float(it["ot1"])
            if "otd" in it:
                fault.otd = float(it["otd"])
            if "oxi" in it:
                fault.oxi = tuple(int(v) for v in it["oxi"])
        elif name == "BC_DYNFLT_NOR" and any(key.endswith("h") for key in it):
            raise ValueError("&BC_DYNFLT_NOR %s (distribution) is not supported by the front end"
                             % [key for key in it if key.endswith("h")])
        elif name == "BC_DYNFLT_SWF":
            fault = fault or Fault()
            fault.swf_kind = int(it.get("kind", 1))
            for key, fname in _SWF_DIST:
                if key in it:
                    fault.values[fname] = float(it[key])
            fault_dists.update(take_dists(k, it, _SWF_DIST))
        elif name == "BC_DYNFLT_RSF":
            fault = fault or Fault()
            fault.rsf_kind = int(it.get("kind", 1))
            for key, fname in _RSF_DIST:
                if key in it:
                    fault.values[fname] = float(it[key])
            fault_dists.update(take_dists(k, it, _RSF_DIST))
        elif name == "BC_DYNFLT_TWF":
            fault = fault or Fault()
            tw = fault.twf or TimeWeakening()
            for key, att in (("kind", "kind"), ("mus", "mus"), ("mud", "mud"), ("mu0", "mu0"), ("x", "X"),
                             ("z", "Z"), ("v", "V"), ("l", "L"), ("t", "T"), ("dc", "Dc")):
                if key in it:
                    setattr(tw, att, type(getattr(tw, att))(it[key]))
            fault.twf = tw
        elif name == "BC_DYNFLT_NOR":
            fault = fault or Fault()
            fault.normal_kind = int(it.get("kind", 1))
            for key, att in (("t", "normal_T"), ("l", "normal_L"), ("v", "normal_V")):
                if key in it:
                    setattr(fault, att, float(it[key]))
        elif name == "TIME":
            time.kind = str(it.get("kind", "leapfrog")).lower()
            if time.kind not in TIME_KINDS:
                raise ValueError("time scheme %s is not on the GPU path" % time.kind)
            if "dt" in it:
                time.dt = float(it["dt"])
            if "courant" in it:
                time.courant = float(it["courant"])
            if "totaltime" in it:
                time.total_time = float(it["totaltime"])
            if "nbsteps" in it:
                time.nsteps = int(it["nbsteps"])
        elif name == "TIME_NEWMARK":
            time.beta = float(it.get("beta", 0.0))
            time.gamma = float(it.get("gamma", 0.5))
        elif name == "TIME_HHTA":
            time.alpha = float(it.get("alpha", 0.5))
            time.rho = float(it.get("rho", 0.5))
        elif name == "SRC_DEF":
            mech = str(it.get("mechanism", "FORCE")).upper()
            if mech not in ("FORCE", "EXPLOSION", "DOUBLE_COUPLE", "MOMENT", "WAVE"):
                raise ValueError("source mechanism %s is not on the GPU path" % mech)
            src = src or Sources(coords=[])
            src.mechanism = mech
            sname = str(it.get("stf", "RICKER")).strip().upper()
            if sname == "RICKER":
                q = k + 1
                while q < len(blocks) and blocks[q][0] != "STF_RICKER":
                    q += 1
                if q < len(blocks):
                    consumed.add(q)
                    r = blocks[q][1]
                    src.f0 = float(r.get("f0", 0.0))
                    src.onset = float(r.get("onset", 0.0))
                    src.ampli = float(r.get("ampli", 1.0))
            else:
                src.stf, _ = take_stf(k, sname)
            if mech == "WAVE":
                # WAVE_read reads the first &SRC_WAVE of the file (src_gen.f90:187-190)
                w = next((b for n_, b in blocks if n_ == "SRC_WAVE"), None)
                if w is None:
                    raise ValueError("WAVE_read: SRC_WAVE input block not found")
                src.wave_angle = float(w.get("angle", 0.0))
                src.wave_phase = str(w.get("phase", "S")).strip().upper()
                if src.wave_phase not in ("P", "S"):
                    raise ValueError("WAVE_read: phase must be S or P")
            f = str(it.get("file", "")).strip()
            if f and f.lower() != "none":
                # one source per line: x, z [, time delay [, relative amplitude]]
                # (SO_read, src_gen.f90:70-79)
                t = np.loadtxt(os.path.join(base or ".", f), ndmin=2)
                n0 = len(src.coords)
                src.coords = list(src.coords) + [(float(r[0]), float(r[1])) for r in t]
                if t.shape[1] > 2 or src.tdelay is not None:
                    td = list(src.tdelay) if src.tdelay is not None else [0.0] * n0
                    src.tdelay = td + [float(r[2]) if t.shape[1] > 2 else 0.0 for r in t]
                if t.shape[1] > 3 or src.relamp is not None:
                    ra = list(src.relamp) if src.relamp is not None else [1.0] * n0
                    src.relamp = ra + [float(r[3]) if t.shape[1] > 3 else 1.0 for r in t]
            else:
                c = it["coord"]
                src.coords = list(src.coords) + [(float(c[0]), float(c[1]))]
                if src.tdelay is not None:
                    src.tdelay = list(src.tdelay) + [0.0]
                if src.relamp is not None:
                    src.relamp = list(src.relamp) + [1.0]
        elif name == "STF_RICKER":
            src = src or Sources(coords=[])
            src.f0 = float(it.get("f0", src.f0))
            src.onset = float(it.get("onset", src.onset))
            src.ampli = float(it.get("ampli", src.ampli))
        elif name == "SRC_MOMENT":
            src = src or Sources(coords=[])
            if "myx" in it or "myz" in it:
                src.M = (float(it.get("myx", 0.0)), float(it.get("myz", 0.0)), 0.0, 0.0)
            else:
                src.M = tuple(float(it.get(k, 0.0)) for k in ("mxx", "mxz", "mzx", "mzz"))
        elif name == "SRC_DOUBLE_COUPLE":
            src = src or Sources(coords=[])
            src.dip = float(it.get("dip", 90.0))
        elif name == "SRC_FORCE":
            src = src or Sources(coords=[])
            src.angle = float(it.get("angle", 0.0))
        elif name == "REC_LINE":
            rec = Receivers(number=int(it.get("number", 0)))
            f = str(it.get("file", "")).strip()
            if f and f.lower() != "none":
                # station positions, two columns x z (REC_read, receivers.f90:43-44)
                rec.coords = np.loadtxt(os.path.join(base or ".", f), ndmin=2)[:, :2].copy()  # (n, 2)
                rec.number = rec.coords.shape[0]
            if "first" in it:
                rec.first = _pair(it["first"])
            if "last" in it:
                rec.last = _pair(it["last"])
            rec.field = str(it.get("field", "V")).upper()
            rec.isamp = int(it.get("isamp", 1))
            rec.atnode = bool(it.get("atnode", True))
        else:
            deck.skipped.append(name)
        k += 1
    deck.materials = mats
    deck.domains = domains
    deck.absorbing = absorbing
    deck.fault = fault
    deck.time = time
    deck.sources = src
    deck.receivers = rec
    if fault_dists or mat_dists:
        _evaluate(deck, fault_dists, mat_dists)
    return deck


def _evaluate(deck, fault_dists, mat_dists):
    """Distributions at the fault nodes (bc%coord = coord(:, node1),
    bc_dynflt.f90:302) and at the GLL points of the elements of each
    material tag (ngll, ngll, nelem arrays of the deck)."""
    from .api import Grid
    grid = Grid(deck)
    xz = grid.coord()
    if fault_dists:
        if deck.fault is None:
            raise ValueError("fault distributions without a fault")
        n1, _ = grid.fault_nodes()
        x, z = xz[0, n1 - 1], xz[1, n1 - 1]
        for name, dist in fault_dists.items():
            deck.fault.values[name] = dist(x, z)
    if mat_dists:
        ib = grid.ibool() - 1  # (ngll, ngll, nelem)
        tags = grid.tags()
        px, pz = xz[0][ib], xz[1][ib]
        shape = ib.shape
        for m in deck.materials:
            md = mat_dists.get(m.tag)
            if not md:
                continue
            sel = np.broadcast_to(tags == m.tag, shape)
            props = ("rho", "c11", "c13", "c33", "c55", "c66") if m.aniso else ("rho", "cp", "cs")
            for name in props + ("kveta",):
                if name == "kveta" and "kveta" not in md:
                    continue
                arr = deck.hetero.setdefault(name, np.zeros(shape))
                const = m.kv_eta if name == "kveta" else getattr(m, name)
                arr[sel] = md[name](px[sel], pz[sel]) if name in md else const
            m.hetero = True


def _stf_values(sname, b, base):
    """Stf of an &STF_<sname> block, with the reference's defaults
    (stf_gaussian.f90:45-47, stf_brune.f90:43-44, stf_harmonic.f90:41-42,
    stf_user.f90:47-52, stf_tabulated.f90:47-63)."""
    from .deck import Stf
    if sname == "RICKER":
        return Stf("RICKER", f0=float(b.get("f0", 0.0)), onset=float(b.get("onset", 0.0)),
                   ampli=float(b.get("ampli", 1.0)))
    if sname == "GAUSSIAN":
        return Stf("GAUSSIAN", f0=float(b.get("f0", 1.0)), onset=float(b.get("onset", 0.0)),
                   ampli=float(b.get("ampli", 1.0)))
    if sname == "BRUNE":
        return Stf("BRUNE", f0=float(b.get("fc", 1.0)), ampli=float(b.get("ampli", 1.0)))
    if sname == "HARMONIC":
        return Stf("HARMONIC", f0=float(b.get("f0", 0.0)), ampli=float(b.get("ampli", 0.0)))
    if sname == "USER":
        return Stf("USER", onset=float(b.get("onset", 0.0)), ampli=float(b.get("ampli", 1.0)),
                   par1=float(b.get("par1", 0.0)), par2=float(b.get("par2", 0.0)))
    f = str(b.get("file", "stf.tab")).strip()
    t = np.loadtxt(os.path.join(base or ".", f), ndmin=2)
    return Stf("TAB", tab=(t[:, 0].copy(), t[:, 1].copy()))


def load_parinp(path, precision=None):
    """ParDeck for the Par.inp file at `path` (tables named by `file=` in
    &DIST_* blocks are read relative to its folder)."""
    with open(path) as f:
        return deck_from_parinp(f.read(), precision, base=os.path.dirname(os.path.abspath(path)))
