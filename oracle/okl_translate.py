"""OKL -> C translation of single reference kernels (test infrastructure only).

The reference's device code is OKL, which only OCCA translates; OCCA itself is an
empty submodule in the reference tree. This script does what OCCA's Serial/OpenMP
backends do for the kernels it is given, so that the reference's own kernel text can
be compiled with gcc and used as the CPU baseline and as a checker of the oracle:

  * @kernel void name(...)          -> void <prefix>name(...)
  * for(init; cond; inc; @outer(d))  -> for(init; cond; inc); the @outer(0) loop gets
                                        "#pragma omp parallel for" (OpenMP mode)
  * for(init; cond; inc; @inner(d))  -> for(init; cond; inc); consecutive inner nests run
                                        one after the other, which is the barrier between them
  * @shared T a[n]                   -> T a[n]   (local to one outer iteration)
  * @exclusive T a[n], b             -> T a[I1][I0][n], b[I1][I0], every use indexed by the
                                        inner loop variables ([j][i] for @inner(1) j, @inner(0) i)
  * @restrict T *p                  -> T * restrict p;  @barrier -> (nothing);  #pragma unroll -> (nothing)

Kernel source is read from the reference tree at build time (LIBPARANUMAL_DIR, or the
path given) and the generated C goes to oracle/_ref/ only; nothing of the reference is
committed. Usage: python okl_translate.py <libParanumal source tree>
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
GENERATED = os.path.join(REF_DIR, "ref_kernels.c")

# (OKL file within the reference tree, kernel name, exported C name, kernel defines)
KERNELS = [
    # solvers/elliptic/okl/ellipticAxHex3D.okl:156-295 (ellipticPartialAxHex3D = _v0); the
    # geometric-factor defines are meshGeometricFactorsHex3D.cpp:70-85's
    ("solvers/elliptic/okl/ellipticAxHex3D.okl", "ellipticPartialAxHex3D_v0", "ref_partialAxHex3D_N%d",
     {"p_Nggeo": 6, "p_G00ID": 0, "p_G01ID": 1, "p_G02ID": 2, "p_G11ID": 3, "p_G12ID": 4, "p_G22ID": 5}),
    # libs/ogs/okl/ogsKernels.okl:86-122 with the Add/double defines of ogsUtils.cpp:53-110
    # and ogsOperator.hpp:122-123 (blockSize 256, gatherNodesPerBlock 512)
    ("libs/ogs/okl/ogsKernels.okl", "gather", "ref_ogsGatherAdd",
     {"T": "double", "OGS_OP_INIT": "0.0", "OGS_OP(a,b)": "a+=b", "p_blockSize": 256,
      "p_gatherNodesPerBlock": 512}),
]
DEGREES = range(1, 9)


def strip_comments(s):
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", "", s)


def extract_kernel(src, name):
    m = re.search(r"@kernel\s+void\s+%s\s*\(" % re.escape(name), src)
    if not m:
        raise ValueError("kernel %s not found" % name)
    i = src.index("{", m.end())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[m.start():j + 1]
    raise ValueError("unbalanced braces in %s" % name)


LOOP = re.compile(r"for\s*\(([^;]*);([^;]*);([^;]*);\s*@(outer|inner)\s*\(\s*(\d)\s*\)\s*\)")


def translate(kernel, cname):
    k = strip_comments(kernel)
    k = re.sub(r"@kernel\s+void\s+\w+\s*\(", "void %s(" % cname, k, count=1)
    k = re.sub(r"#pragma\s+unroll[^\n]*", "", k)
    # OCCA puts the qualifier on the pointer: @restrict const T *p -> const T * restrict p
    k = re.sub(r"@restrict\s+([^,()*]*?)\*\s*(\w+)", r"\1* restrict \2", k)
    k = k.replace("@shared", "")
    k = re.sub(r"@barrier\s*\(?[^;]*\)?\s*;", ";", k)
    # inner loop variables and extents, outermost first (every inner nest of a kernel uses
    # the same variables)
    inner = {}
    for m in LOOP.finditer(k):
        if m.group(4) == "inner":
            var = re.search(r"(\w+)\s*=", m.group(1)).group(1)
            ext = re.search(r"<\s*(.+)$", m.group(2).strip()).group(1).strip()
            inner[int(m.group(5))] = (var, ext)
    dims = [inner[d] for d in sorted(inner, reverse=True)]
    idx = "".join("[%s]" % v for v, _ in dims)
    ext = "".join("[%s]" % e for _, e in dims)

    def loop(m):
        head = "for(%s;%s;%s)" % (m.group(1), m.group(2), m.group(3))
        if m.group(4) == "outer" and m.group(5) == "0":
            return "\n#pragma omp parallel for\n" + head
        return head
    k = LOOP.sub(loop, k)
    # @exclusive declarations: one private copy per inner-loop thread
    names = []

    def excl(m):
        typ, decls = m.group(1), m.group(2)
        out = []
        for d in decls.split(","):
            d = d.strip()
            nm = re.match(r"(\w+)", d).group(1)
            names.append(nm)
            out.append(nm + ext + d[len(nm):])
        return "%s %s;" % (typ, ", ".join(out))
    k = re.sub(r"@exclusive\s+(\w+)\s+([^;]+);", excl, k)
    body_start = k.index("{")
    head, body = k[:body_start], k[body_start:]
    for nm in names:
        # every use of an exclusive name (declarations carry the extents, not the indices)
        body = re.sub(r"\b%s\b(?!%s)" % (nm, re.escape(ext)), nm + idx, body)
    if re.search(r"@\w+", head + body):
        raise ValueError("untranslated attribute in %s: %s" % (cname, re.search(r"@\w+", head + body).group(0)))
    return head + body


def generate(ref_root, out=GENERATED):
    parts = ["/* Generated by oracle/okl_translate.py from the reference's OKL kernels\n"
             " * (OCCA Serial/OpenMP semantics). Test infrastructure; not committed. */\n",
             "#include <stdint.h>\n", "typedef double dfloat;\ntypedef int dlong;\ntypedef long long hlong;\n"]
    for path, name, cname, defs in KERNELS:
        src = open(os.path.join(ref_root, path)).read()
        kern = extract_kernel(src, name)
        degrees = DEGREES if "%d" in cname else [None]
        for N in degrees:
            d = dict(defs)
            if N is not None:
                Nq = N + 1
                d.update({"p_N": N, "p_Nq": Nq, "p_Np": Nq ** 3})
            parts.append("\n/* %s:%s%s */\n" % (path, name, "" if N is None else " at N=%d" % N))
            parts += ["#define %s %s\n" % (kk, v) for kk, v in d.items()]
            parts.append(translate(kern, cname % N if N is not None else cname) + "\n")
            parts += ["#undef %s\n" % kk.split("(")[0] for kk in d]
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        f.write("".join(parts))
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LIBPARANUMAL_DIR")
    if not root:
        sys.exit("usage: okl_translate.py <libParanumal source tree> (or set LIBPARANUMAL_DIR)")
    print(generate(root))
