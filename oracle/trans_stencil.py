"""Builds the oracle of the trans_sim coefficient-change path (test
infrastructure only): the reference's own transformed-frame stencil, computed
by its generated functions (src/stenc_funcs.hh) exactly as
trans_sim_3d::set_up_stencil_and_matrices (src/trans_sim_3d.cpp:1187-1489)
calls them.

The case -> function table is read from that switch in the reference source
(so whatever it assigns, it assigns here too), written to
oracle/_ref/trans_stencil_gen.cc, and compiled with the reference's
stenc_funcs.hh into oracle/_ref/libtransstencil.so.  Needs the reference
checkout; run

    python oracle/trans_stencil.py <reference checkout>/src

The library exports
    void ref_trans_stencil(const double *T, double mu, double lamb,
                           double dx, double dy, double dz, double dt,
                           double *stencil /* 27*9 */, double *fix /* 9 */)
with T row-major (a11 .. a33) and D = T.det() (src/mat3.hh:169-171).
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def parse_switch(src):
    text = open(os.path.join(src, "trans_sim_3d.cpp")).read()
    start = text.index("void trans_sim_3d::set_up_stencil_and_matrices")
    end = text.index("mgrid.setup_matrices(*this)", start)
    body = text[start:end]
    cases = {}
    cur = None
    for line in body.splitlines():
        m = re.match(r"\s*case\s+(\d+)\s*:", line)
        if m:
            cur = int(m.group(1))
            cases[cur] = []
            continue
        m = re.match(r"\s*st([1-3])([1-3])\s*=\s*([A-Za-z_0-9]+)\s*\(", line)
        if m and cur is not None:
            cases[cur].append((int(m.group(1)), int(m.group(2)), m.group(3)))
    return cases


def generate(cases):
    args = "t11, t12, t13, t21, t22, t23, t31, t32, t33, mu, lamb, D, dx, dy, dz"
    lines = ['#include "stenc_funcs.hh"', "", 'extern "C" void ref_trans_stencil(const double *T, double mu, '
             "double lamb, double dx, double dy, double dz, double dt, double *out, double *fix) {",
             "    const double t11 = T[0], t12 = T[1], t13 = T[2], t21 = T[3], t22 = T[4], t23 = T[5],",
             "                 t31 = T[6], t32 = T[7], t33 = T[8];",
             "    const double D = t11 * (t22 * t33 - t23 * t32) + t21 * (t13 * t32 - t12 * t33) + "
             "t31 * (t12 * t23 - t13 * t22);",
             "    for (int e = 0; e < 243; e++) out[e] = 0.0;"]
    for c, assigns in sorted(cases.items()):
        lines.append("    {")
        lines.append("        double st[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};")
        for r, col, fn in assigns:
            lines.append(f"        st[{3 * (r - 1) + col - 1}] = {fn}({args});")
        lines.append(f"        for (int e = 0; e < 9; e++) out[9 * {c} + e] = -dt * st[e];")
        lines.append("    }")
    lines += ["    const double f = -dt * 2 * ((lamb + 2 * mu) / dx / dx + mu / dy / dy + mu / dz / dz);",
              "    for (int e = 0; e < 9; e++) fix[e] = (e % 4 == 0) ? f : 0.0;", "}", ""]
    return "\n".join(lines)


def main():
    if len(sys.argv) > 1:
        src = sys.argv[1]
    else:
        src = os.path.join(os.environ.get("STZPP_REFERENCE", "/root/reference"), "src")
    if not os.path.exists(os.path.join(src, "stenc_funcs.hh")):
        sys.exit(f"reference sources not found at {src}")
    cases = parse_switch(src)
    if len(cases) != 19:
        sys.exit(f"expected 19 stencil cases, found {len(cases)}")
    os.makedirs(OUT, exist_ok=True)
    gen = os.path.join(OUT, "trans_stencil_gen.cc")
    with open(gen, "w") as f:
        f.write(generate(cases))
    lib = os.path.join(OUT, "libtransstencil.so")
    subprocess.run(["g++", "-O2", "-std=c++11", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-I", src, "-o", lib,
                    gen], check=True)
    print("built", lib, "cases", sorted(cases))


if __name__ == "__main__":
    main()
