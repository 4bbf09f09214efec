"""The FP32-arithmetic physics build (gen_f32.py): the transformation of
the FP64 kernel sources, checked on the text (no GPU).  The build itself
compiles the result; the GPU tests bound its per-field error."""
import re
from pathlib import Path

from fortranutils_gb300 import gen_f32

CSRC = Path(gen_f32.__file__).resolve().parent / "csrc"


def test_generated_sources(tmp_path):
    outs = gen_f32.generate(CSRC, tmp_path)
    assert [p.name for p in outs] == ["k_phys_f32.cu", "k_sgs_f32.cu"]
    for p in outs:
        text = p.read_text()
        assert "#define LES_F32_PHYS 1" in text
        # every kernel's FP64 scalar parameter keeps its FP64 type (a
        # cooperative launch passes arguments by address) and is read
        # through an FP32 copy
        for sig, body in re.findall(r"(__global__[^{]*)\{([^\n]*)", text):
            for name in re.findall(r"\bdouble\s+(\w+)_fp64\b", sig):
                assert f"const real {name} = (real){name}_fp64;" in body, name
            assert not re.search(r"\bdouble\s+(?!\w+_fp64)\w+\s*[,)]", sig), sig
        # L2 loads of the sweep convert; no floating literal stays FP64
        assert "__ldcg(" not in text.split("namespace LES_PHYS_NS")[1]
        for span in re.findall(r"__global__.*?\n}\n", text, flags=re.S):
            assert not re.search(r"(?<![\w.])\d+\.\d*(?:[eE][-+]?\d+)?(?![\w.f])", span)


def test_fp64_builds_untouched(tmp_path):
    """The exact and fast builds compile the sources as written."""
    before = {n: (CSRC / n).read_text() for n in ("k_phys.cu", "k_sgs.cu")}
    gen_f32.generate(CSRC, tmp_path)
    for n, t in before.items():
        assert (CSRC / n).read_text() == t


def test_transform_units():
    src = """namespace LES_PHYS_NS {
__global__ void k(const double *__restrict__ a, double *__restrict__ o, double s, int n)
{
    const double *b = a + 1, *c = a + 2;
    double t = 0.5 * (a[0] + b[1]) + s * c[2] + A_.x[3] + F.y[4];
    A_.z[n] = t;
    o[n] = 1.e-30 + 2.0 * t;
}
void host(double d) { double e = d * 0.5; }
}
"""
    out = gen_f32.transform(src, "t.cu")
    assert "LdF a" in out and "double *__restrict__ o" in out
    # a <<<>>> kernel takes its FP64 scalars as float (converted at the launch)
    assert "real s, int n" in out and "s_fp64" not in out
    # a cooperative kernel keeps them double and converts once in its body
    coop = gen_f32.transform(src.replace("void k(", "void k_sc1_sweep("), "t.cu")
    assert "double s_fp64" in coop and "const real s = (real)s_fp64;" in coop
    assert "const LdF b = a + 1, c = a + 2;" in out
    assert "real t = 0.5f * (a[0] + b[1]) + s * c[2] + LdF(A_.x)[3] + LdF(F.y)[4];" in out
    assert "A_.z[n] = t;" in out and "1.e-30f + 2.0f * t" in out
    # host code as written
    assert "void host(double d) { double e = d * 0.5; }" in out


def test_metric_tables_read_as_fp32_copies():
    """Metric tables (the host passes FP32 copies) are read through LdM,
    fields through LdF -- in members, parameters and local views."""
    src = """namespace LES_PHYS_NS {
__global__ void k(const double *__restrict__ u, const double *__restrict__ dip, double s)
{
    const double *dkp = A_.dkp + b.off1k, *w = A_.w;
    double t = u[0] * dip[1] + A_.diu[2] + A_.rho[3] + dkp[4] + w[5] + A_.m[q][6];
}
}
"""
    out = gen_f32.transform(src, "t.cu")
    assert "LdF u" in out and "LdM dip" in out
    assert "const LdM dkp = LdM(A_.dkp) + b.off1k; const LdF w = A_.w;" in out
    assert "LdM(A_.diu)[2]" in out and "LdF(A_.rho)[3]" in out and "LdM(A_.m[q])[6]" in out
