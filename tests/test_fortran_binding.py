"""The Fortran binding (fortran-mpi-fdtd_gb300/fortran/fdtd_gpu_mod.f90) and
the ctypes binding (fdtd_gpu/abi.py, job.py) checked mechanically against the
C header: every entry point has a bind(c) interface with the header's binding
label, its arguments in the same order with the same names, each passed by
value or by reference as the C type says, with the matching interoperable
kind; every descriptor is a bind(c) derived type (and a ctypes Structure)
with the header's fields in the header's order and kinds; and the named
constants agree.  No Fortran compiler is needed (none is installed), so the
check parses the sources.  The last tests change the header in memory and
see the check fail."""
import ctypes as C
import os
import re

import pytest

from fdtd_gpu import abi, job

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fdtd_gb300.h")
FMOD = os.path.join(ROOT, "fortran-mpi-fdtd_gb300", "fortran", "fdtd_gpu_mod.f90")
FTYPES = os.path.join(ROOT, "fortran-mpi-fdtd_gb300", "fortran", "fdtd_gpu_types.f90")

# C scalar type -> the iso_c_binding kind of the same size and representation
CKIND = {"int32_t": "integer(c_int32_t)", "int": "integer(c_int)", "double": "real(c_double)",
         "int64_t": "integer(c_int64_t)", "uint64_t": "integer(c_int64_t)", "size_t": "integer(c_size_t)",
         "char": "character(kind=c_char)", "uint8_t": "integer(c_int8_t)"}
OPAQUE = {"fdtd_job", "fdtd_server"}


# ---- the C header --------------------------------------------------------------
def _strip_c(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def c_defines(text):
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(\w+)\s+(\d+)\s*$", text, re.M)}


def c_enums(text):
    out = {}
    for body in re.findall(r"enum\s*\{(.*?)\}", text, re.S):
        for item in body.split(","):
            m = re.match(r"\s*(\w+)\s*=\s*(-?\d+)\s*$", item)
            if m:
                out[m.group(1)] = int(m.group(2))
    return out


def c_structs(text):
    """name -> [(field, ctype, is_pointer, dims)]"""
    text = _strip_c(text)
    defs = c_defines(text)
    out = {}
    for m in re.finditer(r"typedef\s+struct\s*\w*\s*\{(.*?)\}\s*(\w+)\s*;", text, re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            mt = re.match(r"(const\s+)?(\w+)\s+(.*)$", decl)
            ctype, rest = mt.group(2), mt.group(3)
            for item in rest.split(","):
                item = item.strip()
                ptr = item.startswith("*")
                mi = re.match(r"\*?\s*(\w+)\s*((?:\[\s*\w+\s*\])*)$", item)
                dims = [int(defs.get(d, d)) for d in re.findall(r"\[\s*(\w+)\s*\]", mi.group(2))]
                fields.append((mi.group(1), ctype, ptr, dims))
        out[m.group(2)] = fields
    return out


def c_functions(text):
    """name -> [(param, ctype, pointer depth, dims)]"""
    text = _strip_c(text)
    out = {}
    for m in re.finditer(r"^int\s+(fdtd_\w+)\s*\((.*?)\)\s*;", text, re.S | re.M):
        params = []
        for p in m.group(2).split(","):
            p = " ".join(p.split())
            mp = re.match(r"(?:const\s+)?(\w+)\s*(\**)\s*(\w+)\s*((?:\[\s*\w+\s*\])*)$", p)
            assert mp, p
            dims = [int(d) for d in re.findall(r"\[\s*(\d+)\s*\]", mp.group(4))]
            params.append((mp.group(3), mp.group(1), len(mp.group(2)), dims))
        out[m.group(1)] = params
    return out


# ---- the Fortran module ------------------------------------------------------------
def _fortran_statements(text):
    lines = []
    for ln in text.splitlines():
        ln = re.sub(r"!.*$", "", ln).rstrip()
        if lines and lines[-1].endswith("&"):
            lines[-1] = lines[-1][:-1] + " " + ln.strip().lstrip("&")
        else:
            lines.append(ln)
    out = []
    for ln in lines:
        out.extend(s.strip() for s in ln.split(";") if s.strip())
    return out


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts if p.strip()]


def _decl(stmt):
    """'integer(c_int32_t), intent(out) :: a, b(3)' -> (kind, attrs, [(name, dims)])"""
    spec, names = stmt.split("::", 1)
    sp = _split_top(spec)
    kind, attrs = sp[0].replace(" ", "").lower(), [a.replace(" ", "").lower() for a in sp[1:]]
    ents = []
    for e in _split_top(names):
        e = e.split("=")[0].strip()
        me = re.match(r"(\w+)\s*(?:\((.*)\))?$", e)
        dims = [d.strip() for d in me.group(2).split(",")] if me.group(2) else []
        ents.append((me.group(1), dims))
    return kind, attrs, ents


def f_module(text):
    stmts = _fortran_statements(text)
    types, funcs, params = {}, {}, {}
    i = 0
    while i < len(stmts):
        s = stmts[i]
        low = s.lower()
        mt = re.match(r"type\s*,\s*bind\s*\(\s*c\s*\)\s*::\s*(\w+)$", low)
        mf = re.match(r"integer\s*\(\s*c_int\s*\)\s+function\s+(\w+)\s*\((.*?)\)\s*bind\s*\(\s*c\s*(?:,\s*name\s*=\s*'(\w+)')?\s*\)$",
                      s, re.I)
        if mt:
            comps = []
            i += 1
            while not stmts[i].lower().startswith("end type"):
                kind, attrs, ents = _decl(stmts[i])
                comps.extend((n.lower(), kind, dims) for n, dims in ents)
                i += 1
            types[mt.group(1)] = comps
        elif mf:
            name, args = mf.group(1), [a.strip().lower() for a in mf.group(2).split(",") if a.strip()]
            label = mf.group(3) or name.lower()
            decl = {}
            i += 1
            while not stmts[i].lower().startswith("end function"):
                if not stmts[i].lower().startswith("import"):
                    kind, attrs, ents = _decl(stmts[i])
                    for n, dims in ents:
                        decl[n.lower()] = (kind, "value" in attrs, dims)
                i += 1
            funcs[label] = [(a,) + decl[a] for a in args]
        elif "parameter" in low and "::" in low:
            for e in _split_top(s.split("::", 1)[1]):
                mp = re.match(r"(\w+)\s*=\s*(-?\d+)$", e.strip())
                if mp:
                    params[mp.group(1)] = int(mp.group(2))
        i += 1
    return types, funcs, params


def check_binding(header_text, fortran_text):
    """All mismatches between the header and the Fortran module, as messages."""
    errs = []
    structs, funcs = c_structs(header_text), c_functions(header_text)
    consts = dict(c_enums(_strip_c(header_text)), **c_defines(_strip_c(header_text)))
    ftypes, ffuncs, fparams = f_module(fortran_text)
    # descriptors
    for sname, fields in structs.items():
        if sname not in ftypes:
            errs.append(f"struct {sname}: no bind(c) derived type")
            continue
        want = [(f, "type(c_ptr)" if ptr else CKIND[t], [str(d) for d in reversed(dims)]) for f, t, ptr, dims in fields]
        got = ftypes[sname]
        if [w[0] for w in want] != [g[0] for g in got]:
            errs.append(f"struct {sname}: fields {[g[0] for g in got]} != {[w[0] for w in want]}")
            continue
        for w, g in zip(want, got):
            if w != g:
                errs.append(f"struct {sname}.{w[0]}: Fortran {g[1:]} != C {w[1:]}")
    for t in ftypes:
        if t not in structs:
            errs.append(f"derived type {t}: no such struct in the header")
    # entry points
    for fname, cparams in funcs.items():
        if fname not in ffuncs:
            errs.append(f"{fname}: no bind(c) interface with this label")
            continue
        fp = ffuncs[fname]
        if [p[0] for p in cparams] != [p[0] for p in fp]:
            errs.append(f"{fname}: arguments {[p[0] for p in fp]} != {[p[0] for p in cparams]}")
            continue
        for (pn, ct, depth, dims), (_, kind, value, fdims) in zip(cparams, fp):
            where = f"{fname}({pn})"
            if depth == 0 and not dims:                          # a scalar by value
                if not value or kind != CKIND[ct]:
                    errs.append(f"{where}: C {ct} by value, Fortran {kind} value={value}")
            elif ct in OPAQUE:                                   # a handle, or its address
                if kind != "type(c_ptr)" or value != (depth == 1):
                    errs.append(f"{where}: C {ct}{'*' * depth}, Fortran {kind} value={value}")
            elif ct in structs:                                  # a descriptor by reference
                if kind != f"type({ct})" or value or depth != 1:
                    errs.append(f"{where}: C {ct}*, Fortran {kind} value={value}")
            elif ct == "void":                                   # an address: c_ptr by value, or any array
                if not ((kind == "type(c_ptr)" and value) or (not value and fdims == ["*"])):
                    errs.append(f"{where}: C void*, Fortran {kind} value={value} dims={fdims}")
            else:                                                # a scalar or array by reference
                ok_ref = kind == CKIND[ct] and not value and depth + len(dims) == 1
                ok_ptr = kind == "type(c_ptr)" and value and depth == 1
                if not (ok_ref or ok_ptr):
                    errs.append(f"{where}: C {ct}{'*' * depth}{dims}, Fortran {kind} value={value}")
                elif dims and ok_ref and fdims != [str(d) for d in dims]:
                    errs.append(f"{where}: C dims {dims}, Fortran {fdims}")
    for f in ffuncs:
        if f not in funcs:
            errs.append(f"interface {f}: no such entry point in the header")
    # named constants
    for n, v in fparams.items():
        if n in consts and consts[n] != v:
            errs.append(f"parameter {n} = {v}, header {consts[n]}")
    for n in consts:
        if n.startswith("FDTD_") and n not in fparams and not n.endswith("_H") and n != "FDTD_NOALLOC_STAGE_BYTES":
            errs.append(f"constant {n}: no Fortran parameter")
    return errs


def test_fortran_module_matches_header():
    errs = check_binding(open(HEADER).read(), open(FMOD).read())
    assert not errs, "\n".join(errs)


def test_fortran_wrappers_use_declared_entry_points():
    """The type-bound wrappers call only entry points the module declares,
    with as many arguments as the interface takes."""
    _, ffuncs, _ = f_module(open(FMOD).read())
    text = re.sub(r"!.*", "", open(FTYPES).read())
    names = {f.lower(): f for f in ffuncs}
    for m in re.finditer(r"\b(fdtd_\w+)\s*\(", text):
        key = m.group(1).lower()
        if key in ("fdtd_gpu_mod", "fdtd_gpu_types") or key in {t for t in c_structs(open(HEADER).read())}:
            continue
        assert key in names, m.group(1)
        depth, j = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(text[j], 0)
            j += 1
        nargs = len(_split_top(text[m.end():j - 1]))
        assert nargs == len(ffuncs[names[key]]), (m.group(1), nargs)


CTYPES = {"fdtd_grid_desc": abi.GridDesc, "fdtd_region": abi.Region, "fdtd_drude2cp": abi.Drude2CP,
          "fdtd_graphene_desc": abi.GrapheneDesc, "fdtd_tfsf_desc": abi.TfsfDesc,
          "fdtd_lorentz_desc": abi.LorentzDesc, "fdtd_graphene_nk_desc": abi.GrapheneNkDesc,
          "fdtd_graphene_cp_desc": abi.GrapheneCpDesc, "fdtd_pml_desc": abi.PmlDesc,
          "fdtd_source_desc": abi.SourceDesc, "fdtd_monitor_desc": abi.MonitorDesc,
          "fdtd_probe_desc": abi.ProbeDesc, "fdtd_tfsf1d_desc": abi.Tfsf1dDesc,
          "fdtd_server_desc": abi.ServerDesc, "fdtd_server_status": abi.ServerStatus}
CTY = {"int32_t": C.c_int32, "double": C.c_double, "int64_t": C.c_int64, "uint64_t": C.c_uint64}


def _ctypes_field(t):
    dims = []
    while hasattr(t, "_length_"):
        dims.append(t._length_)
        t = t._type_
    return t, dims


def test_ctypes_structs_match_header():
    structs = c_structs(open(HEADER).read())
    assert set(structs) == set(CTYPES), set(structs) ^ set(CTYPES)
    for name, fields in structs.items():
        got = CTYPES[name]._fields_
        assert [g[0] for g in got] == [f[0] for f in fields], name
        for (fname, ctype, ptr, dims), (_, t) in zip(fields, got):
            if ptr:
                assert issubclass(t, C._Pointer), (name, fname)
                continue
            base, tdims = _ctypes_field(t)
            assert base is CTY[ctype] and tdims == dims, (name, fname, base, tdims)


def test_ctypes_signatures_match_header():
    """job.py's argtypes: one per C parameter, pointers as pointers, scalars
    as the C scalar's ctypes type."""
    funcs = c_functions(open(HEADER).read())
    L = job.lib() if os.path.exists(job.LIB_PATH) else pytest.skip("library not built")
    scal = {"int32_t": C.c_int32, "double": C.c_double, "uint64_t": C.c_uint64, "int64_t": C.c_int64,
            "size_t": C.c_size_t}
    for name, params in funcs.items():
        at = getattr(L, name).argtypes
        assert len(at) == len(params), name
        for (pn, ct, depth, dims), t in zip(params, at):
            if depth == 0 and not dims:
                assert t is scal[ct], (name, pn, t)
            else:
                assert t in (C.c_void_p, C.c_char_p) or issubclass(t, C._Pointer), (name, pn, t)


@pytest.mark.parametrize("change", ["rename_field", "reorder_fields", "drop_value", "kind"])
def test_check_catches_a_changed_header(change):
    """The check is not vacuous: a header whose descriptor field is renamed
    or reordered, or whose entry point takes an argument differently, no
    longer matches the Fortran module."""
    h = open(HEADER).read()
    if change == "rename_field":
        h2 = h.replace("double eps_line;", "double eps_ln;")
    elif change == "reorder_fields":
        h2 = h.replace("  double eps_lo, eps_hi;/* relative", "  double eps_hi, eps_lo;/* relative")
    elif change == "drop_value":
        h2 = h.replace("int fdtd_sample(fdtd_job *job, int32_t n);", "int fdtd_sample(fdtd_job *job, int32_t *n);")
    else:
        h2 = h.replace("int fdtd_step(fdtd_job *job, int32_t n_first, int32_t n_steps);",
                       "int fdtd_step(fdtd_job *job, int64_t n_first, int32_t n_steps);")
    assert h2 != h
    assert check_binding(h2, open(FMOD).read())
