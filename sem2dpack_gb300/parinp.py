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
                kind 'DYNFLT' + &BC_DYNFLT / _SWF / _RSF / _TWF / _NOR with
                scalar values (bc_dynflt*.f90)
  &TIME         kind, Dt, Courant, TotalTime, NbSteps + &TIME_NEWMARK
                beta, gamma (time.f90:122-315)
  &SRC_DEF      stf='RICKER', mechanism='FORCE', coord + &STF_RICKER f0,
                onset, ampli + &SRC_FORCE angle (src_gen.f90, stf_ricker.f90)
  &REC_LINE     number, first, last, field, isamp, AtNode (receivers.f90)

and names the blocks it skips in ``deck.skipped``: plots, snapshots,
energies, and the option blocks the reference would not read for this deck
(as it does, a &SRC_WAVE next to a mechanism='FORCE' source, or a
&MESH_EMC2 under method='CARTESIAN', is ignored).  A selecting block that
asks for something off the GPU path (another mesher, material kind,
boundary kind, source mechanism or time scheme, Stacey absorption, a
distribution of fault values) raises ValueError.
"""
import re

from .deck import Fault, Material, ParDeck, Receivers, Sources, TimeWeakening, Time

__all__ = ["read_namelists", "deck_from_parinp", "load_parinp"]

TIME_KINDS = ("leapfrog", "newmark")

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
    toks = _TOKEN.findall(_strip_comments(text))
    blocks, k = [], 0
    while k < len(toks):
        if toks[k] != "&" or k + 1 >= len(toks):
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
        blocks.append((name, items))
        k += 1
    return blocks


def _pair(v):
    return (float(v[0]), float(v[1]))


def deck_from_parinp(text, precision=None):
    """ParDeck for the Par.inp text (see the module docstring)."""
    blocks = read_namelists(text)
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
        if name == "GENERAL":
            deck.ngll = int(it.get("ngll", deck.ngll))
            deck.ndof = int(it.get("ndof", deck.ndof))
            deck.fmax = float(it.get("fmax", deck.fmax))
            if float(it.get("w", 0.0) or 0.0) > 0.0:
                deck.width = float(it["w"])
        elif name == "MESH_DEF":
            if str(it.get("method", "CARTESIAN")).upper() != "CARTESIAN":
                raise ValueError("only &MESH_DEF method='CARTESIAN' is on the GPU path")
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
            j = k + 1
            while j < len(blocks) and blocks[j][0] in ("MAT_ELASTIC", "MAT_KV"):
                bn, b = blocks[j]
                if bn == "MAT_ELASTIC":
                    if "c11" in b:
                        m.aniso = True
                        for c in ("c11", "c13", "c33", "c55", "c66"):
                            setattr(m, c, float(b.get(c, 0.0)))
                        m.rho = float(b.get("rho", 0.0))
                    else:
                        m.rho, m.cp, m.cs = float(b["rho"]), float(b["cp"]), float(b["cs"])
                else:
                    m.kv_eta = float(b.get("eta", 0.0))
                    m.kv_etaxdt = bool(b.get("etaxdt", True))
                j += 1
            mats.append(m)
            k = j
            continue
        elif name == "BC_DEF":
            kind = str(it.get("kind", "")).upper()
            tags = it.get("tags", it.get("tag"))
            tags = [tags] if not isinstance(tags, list) else tags
            cur_bc = kind
            if kind == "ABSORB":
                absorbing.extend(int(t) for t in tags)
                if nxt[0] == "BC_ABSORB" and nxt[1].get("stacey", False):
                    deck.stacey.extend(int(t) for t in tags)
            elif kind == "DYNFLT":
                fault = fault or Fault()
                # a single tag is a one-sided fault: tags = (tag, 0) (bc_gen.f90:126-133)
                fault.tags = (int(tags[0]), int(tags[1]) if len(tags) > 1 else 0)
                deck.fault_first = not absorbing
            elif kind == "DIRNEU":
                b = nxt[1] if nxt[0] == "BC_DIRNEU" else {}
                extra = set(b) - {"h", "v"}
                if extra:
                    raise ValueError("&BC_DIRNEU %s (traction time functions) is not on the GPU path"
                                     % ", ".join(sorted(extra)))
                h, v = str(b.get("h", "N")).upper(), str(b.get("v", "N")).upper()
                deck.dirneu.extend((int(t), h, v, fault is None) for t in tags)
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
            for key, fname in (("tn", "Tn"), ("tt", "Tt"), ("v", "V"), ("sxx", "Sxx"), ("sxy", "Sxy"),
                               ("sxz", "Sxz"), ("syz", "Syz"), ("szz", "Szz"), ("cohesion", "cohesion")):
                if key in it:
                    fault.values[fname] = float(it[key])
            if "ot1" in it:
                fault.ot1 = float(it["ot1"])
            if "otd" in it:
                fault.otd = float(it["otd"])
            if "oxi" in it:
                fault.oxi = tuple(int(v) for v in it["oxi"])
            for key in it:
                if key.endswith("h") and key[:-1] in ("tn", "tt", "v", "sxx", "sxy", "sxz", "syz", "szz"):
                    raise ValueError("&BC_DYNFLT %s (distribution) is not supported by the front end" % key)
        elif name in ("BC_DYNFLT_SWF", "BC_DYNFLT_RSF", "BC_DYNFLT_NOR") and \
                any(key.endswith("h") and len(key) > 1 for key in it if key not in ("h",)):
            bad = [key for key in it if key.endswith("h")]
            raise ValueError("&%s %s (distribution) is not supported by the front end" % (name, bad))
        elif name == "BC_DYNFLT_SWF":
            fault = fault or Fault()
            fault.swf_kind = int(it.get("kind", 1))
            for key, fname in (("dc", "swf_dc"), ("mus", "swf_mus"), ("mud", "swf_mud"), ("p", "swf_p"),
                               ("alpha", "swf_alpha")):
                if key in it:
                    fault.values[fname] = float(it[key])
        elif name == "BC_DYNFLT_RSF":
            fault = fault or Fault()
            fault.rsf_kind = int(it.get("kind", 1))
            for key, fname in (("dc", "rsf_dc"), ("mus", "rsf_mus"), ("a", "rsf_a"), ("b", "rsf_b"),
                               ("vstar", "rsf_vstar"), ("theta", "rsf_theta"), ("vc", "rsf_vc")):
                if key in it:
                    fault.values[fname] = float(it[key])
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
        elif name == "SRC_DEF":
            if str(it.get("stf", "RICKER")).upper() != "RICKER" or \
                    str(it.get("mechanism", "FORCE")).upper() != "FORCE":
                raise ValueError("only RICKER force sources are on the GPU path")
            c = it["coord"]
            src = src or Sources(coords=[])
            src.coords = list(src.coords) + [(float(c[0]), float(c[1]))]
        elif name == "STF_RICKER":
            src = src or Sources(coords=[])
            src.f0 = float(it.get("f0", src.f0))
            src.onset = float(it.get("onset", src.onset))
            src.ampli = float(it.get("ampli", src.ampli))
        elif name == "SRC_FORCE":
            src = src or Sources(coords=[])
            src.angle = float(it.get("angle", 0.0))
        elif name == "REC_LINE":
            rec = Receivers(number=int(it.get("number", 0)))
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
    return deck


def load_parinp(path, precision=None):
    """ParDeck for the Par.inp file at `path`."""
    with open(path) as f:
        return deck_from_parinp(f.read(), precision)
