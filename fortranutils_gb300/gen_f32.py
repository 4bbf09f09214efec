"""Generate the FP32-arithmetic build of the physics kernels.

k_phys.cu and k_sgs.cu (momentum predictors, scalar transport, eddy
viscosity) are written once, in FP64.  This module derives a third build
from them, namespace les_f32, in which every kernel and device function
computes in FP32 while the fields stay FP64 in HBM: each load from an FP64
array is converted on the way in (``LdF``, and ``ldcg_f`` for the L2 loads
of the in-place scalar sweep), stores convert back, locals and
by-value parameters are ``float``, and floating literals carry an ``f``
suffix so that no expression is promoted back to FP64.  Host code (the
launchers) is left as written, so the les_f32 launchers have the same FP64
signatures as les_exact's and les_fast's.  The reciprocal metric tables of
the fast build are used (LES_FAST_PHYS).

The transformation is textual and confined to the bodies of ``__global__``
and ``__device__`` functions; the FP64 builds compile the sources as they
are.  Called by build.py; the output goes to the build directory.
"""
from __future__ import annotations

import re
from pathlib import Path

HEADER = """// Generated by fortranutils_gb300/gen_f32.py from {src}: the FP32-arithmetic
// build (namespace les_f32).  Do not edit; edit {src}.
#define LES_F32_PHYS 1
#define LES_FAST_PHYS 1
"""

# struct members that are not FP64 arrays, or are arrays of pointers
_NOT_FP64 = {"n", "bc", "link", "m", "r", "iststep", "off_ki", "off_jk"}
_STRUCTS = r"(?:A_|F)"
# read-only FP64 arrays the kernels offset before indexing (the 1-D z
# metrics by a block's offset; the scalar in the sweep's L2 loads)
_OFFSET_READ = ("dkp", "dkw", "r_dkp", "r_dkw", "rdkp", "rdkw", "sc1")
# metric tables (struct members and kernel parameters): read through LdM,
# the host passing FP32 copies (phys32_tables); everything else through LdF
_METRICS = {"dip", "diu", "div", "dix", "djp", "dju", "djv", "djx", "rdip", "rdiv", "rdix", "rdjp", "rdju",
            "rdjx", "hijp", "hjip", "hkip", "hkjp", "hiju", "hjiu", "hkiu", "hkju", "hijv", "hjiv", "hkiv",
            "hkjv", "rp", "ru", "rv", "didjp", "rdidjp", "didju", "rdidju", "djdiv", "rdjdiv", "dkp", "dkw",
            "rdkp", "rdkw", "r_dip", "r_diu", "r_dix", "r_djp", "r_dju", "r_djv", "r_djx", "r_rp", "r_dkp",
            "r_dkw", "delta2d", "delta1d"}


# fields that particular kernels read as FP32 copies too (the host converts
# them once per call: each is read by ~7 neighbouring points)
_FIELDS32 = {"k_set_u_int": {"u", "v", "w", "p", "rho", "rhonp1", "gam"},
             "k_set_w_int": {"u", "v", "w", "p", "rho", "rhonp1", "gam"},
             "k_subgrid": {"u", "v", "w", "sc1"}}
_func = ""


def _view(name: str) -> str:
    return "LdM" if name in _METRICS or name in _FIELDS32.get(_func, ()) else "LdF"

_LITERAL = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])")


def _match_close(text: str, i: int, open_c: str, close_c: str) -> int:
    """Index of the bracket closing the one at text[i]."""
    depth = 0
    for j in range(i, len(text)):
        c = text[j]
        if c == open_c:
            depth += 1
        elif c == close_c:
            depth -= 1
            if depth == 0:
                return j
    raise ValueError(f"unbalanced {open_c} at {i}")


def _function_spans(text: str):
    """(start, brace, end) of every __global__ / __device__ function
    definition: start of the qualifier, its body's opening brace, closing
    brace."""
    spans = []
    for m in re.finditer(r"__(?:global|device)__", text):
        start = m.start()
        if spans and start < spans[-1][2]:
            continue  # a qualifier inside an earlier function
        p = text.index("(", m.end())
        q = _match_close(text, p, "(", ")")
        rest = text[q + 1:]
        k = re.match(r"[^;{]*", rest).end()
        if q + 1 + k >= len(text) or text[q + 1 + k] != "{":
            continue  # a declaration
        brace = q + 1 + k
        spans.append((start, brace, _match_close(text, brace, "{", "}")))
    return spans


# kernels launched cooperatively (arguments passed by address as the FP64
# build lays them out): their FP64 scalar parameters stay double
_COOPERATIVE = {"k_sc1_sweep"}


def _params(sig: str):
    """FP64 pointer parameters become converting views (one pointer, the
    same layout).  FP64 scalars become float in device functions and in
    kernels launched with <<<>>> (the launch converts the argument once on
    the host; converting it in every thread would run on GB300's slow FP64
    pipe); in a cooperative kernel they stay double -- the launch passes
    arguments by address, and an FP64 value read as an FP32 parameter is
    garbage -- under a new name, and the body opens with a float copy
    under the old one.  Returns the signature and that opening."""
    sig = re.sub(r"const\s+double\s*\*\s*(?:__restrict__\s*)?(\w+)", lambda m: _view(m.group(1)) + " " + m.group(1),
                 sig)
    if not sig.lstrip().startswith("__global__") or _func not in _COOPERATIVE:
        return re.sub(r"\bdouble\b(?!\s*\*)", "real", sig), ""
    names = re.findall(r"\bdouble\s+(\w+)\s*(?=[,)])", sig)
    sig = re.sub(r"\bdouble\s+(\w+)\s*(?=[,)])", r"double \1_fp64", sig)
    return sig, "".join(f" const real {n} = (real){n}_fp64;" for n in names)


def _member_reads(body: str) -> str:
    """A_.x[...] / F.x[...] reads of FP64 arrays through LdF (not writes)."""
    out, pos = [], 0
    for m in re.finditer(_STRUCTS + r"\.(\w+)\[", body):
        if m.group(1) in _NOT_FP64 or m.start() < pos:
            continue
        close = _match_close(body, m.end() - 1, "[", "]")
        if re.match(r"\s*=(?!=)", body[close + 1:]):
            continue  # a store
        out.append(body[pos:m.start()])
        out.append(_view(m.group(1)) + "(" + body[m.start():m.end() - 1] + ")" + body[m.end() - 1:close + 1])
        pos = close + 1
    out.append(body[pos:])
    return "".join(out)


def _local_pointers(body: str) -> str:
    """`const double *a = ..., *b = ...;` -> `const LdF a = ..., b = ...;`"""
    def fix(m):
        stmt = m.group(0)
        # one declarator per initializer: `*name = A_.member ...`
        parts = re.split(r"(?:^const\s+double\s*\*|,\s*\*)(?=\s*\w+\s*=)", stmt)
        decls = [p.strip() for p in parts if p.strip()]
        views = []
        for d in decls:
            mm = re.search(r"=\s*(?:Ld[FM]\()?(?:A_|F)\.(\w+)", d)
            views.append(_view(mm.group(1)) if mm else "LdF")
        if len(set(views)) == 1:
            return "const " + views[0] + " " + ", ".join(decls)
        return " ".join(f"const {v} {d.rstrip(';')};" for v, d in zip(views, decls))
    return re.sub(r"const\s+double\s*\*(?!\s*const)\s*\w+\s*=[^;]*;", fix, body)


def _body(body: str) -> str:
    # pointer arithmetic on a member goes through the view (which scales
    # the offset for an FP32 copy)
    body = re.sub(_STRUCTS + r"\.(" + "|".join(_OFFSET_READ) + r")(?=\s*\+)",
                  lambda m: _view(m.group(1)) + "(" + m.group(0) + ")", body)
    body = re.sub(r"M\[a\]\[", "LdM(M[a])[", body)
    body = re.sub(r"A_\.(m|r)\[(\w+)\]\[", r"LdM(A_.\1[\2])[", body)
    body = body.replace("__ldcg(", "ldcg_f(")
    body = _local_pointers(body)
    body = _member_reads(body)
    body = re.sub(r"\bdouble\b(?!\s*\*)", "real", body)
    return _LITERAL.sub(lambda m: m.group(1) + "f", body)


def transform(text: str, src: str) -> str:
    spans = _function_spans(text)
    out, pos = [HEADER.format(src=src)], 0
    global _func
    for start, brace, end in spans:
        out.append(text[pos:start])
        _func = [n for n in re.findall(r"(\w+)\s*\(", text[start:brace]) if not n.startswith("__")][0]
        sig, opening = _params(text[start:brace])
        body = _body(text[brace:end + 1])
        out.append(sig)
        out.append(body[0] + opening + body[1:])
        pos = end + 1
    _func = ""
    out.append(text[pos:])
    # macros defined between functions and expanded inside them
    return re.sub(r"^(#define .*)$", lambda m: m.group(1).replace("__ldcg(", "ldcg_f("), "".join(out),
                  flags=re.M)


def generate(csrc: Path, outdir: Path) -> list[Path]:
    """Write k_phys_f32.cu and k_sgs_f32.cu into outdir (only when changed)."""
    outs = []
    for name in ("k_phys.cu", "k_sgs.cu"):
        text = transform((csrc / name).read_text(), name)
        dst = outdir / name.replace(".cu", "_f32.cu")
        if not dst.exists() or dst.read_text() != text:
            dst.write_text(text)
        outs.append(dst)
    return outs
