"""Golden text of the printed line list, from the reference's own printf
sequence (cuda_host.cu:1444-1473).

The format strings are read out of the reference source at run time (the
printf calls of the line printout, in order, skipping commented ones), the
branch letter comes from the reference's own branch() (trove_functions.cpp,
compiled into oracle/_ref/libref.so by oracle/build_ref.sh), and fixed
synthetic field values are formatted with them through the C library's
snprintf, in the reference's order: the header, the class labels and quanta
of the final and the initial level, S, A, I and the level numbers, the
normal-mode quanta, then the transition moments (final degeneracy outer).
Writes tests/golden/line_format_ref.json (fields and text per line).

    REF_DIR=<reference checkout> python tests/golden/make_line_format.py
"""
import ctypes as C
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))

# the conversions each printf of the sequence must carry (a check that the
# extraction found the printout it expects)
EXPECT = ["%4i %4s %4i %4s %1s %11.4f %11.4f %11.4f %3s %3i", "%3s", "", "%3i", "%3s %3i",
          "%3s", "", "%3i", "%16.8e %16.8e %16.8e %6i %6i %8i %8i", "%3i", "", "%3i", "",
          "%16.9e", ""]

CASES = [
    # C2v-like, R branch, one class, three modes, non-degenerate
    dict(jF=3, jI=2, symF="B1", symI="A1", eF=2345.678912, eI=1234.567891, nu=1111.111021,
         cgF=["B1", "A2"], cgI=["A1", "A1"], krotF=2, krotI=1, quantaF=[0, 1, 0, 2],
         quantaI=[0, 0, 1, 0], normalF=[0, 1, 0, 2], normalI=[0, 0, 1, 0], S=1.234567891e-3,
         A=9.87654321e-2, I=4.56789e-21, ilevelF=41, ilevelI=6, ndegF=1, ndegI=1,
         t=[-3.1415926535e-2, 0, 0, 0]),
    # C3v E <- E, Q branch, emission (negative nu printed as |nu|), 2 x 2 moments
    dict(jF=10, jI=10, symF="E", symI="E", eF=500.25, eI=8000.125, nu=-7499.875,
         cgF=["E", "A1", "E"], cgI=["E", "E", "A2"], krotF=10, krotI=0,
         quantaF=[0, 3, 0, 0, 1, 0, 2], quantaI=[0, 0, 0, 1, 0, 0, 0],
         normalF=[0, 3, 0, 0, 1, 0, 2], normalI=[0, 0, 0, 1, 0, 0, 0], S=1.0e-40,
         A=3.3e-35, I=-0.0, ilevelF=123456, ilevelI=0, ndegF=2, ndegI=2,
         t=[1.0e-12, -2.5e-13, 7.77e-20, -1.0]),
    # P branch, 2 x 1 moments, rounding at the printed precision, large numbers
    dict(jF=39, jI=40, symF="A2", symI="E", eF=11999.99995, eI=11999.99994, nu=-0.00001,
         cgF=["A2"], cgI=["E"], krotF=39, krotI=40, quantaF=[0, 12, 7], quantaI=[0, 11, 8],
         normalF=[0, 12, 7], normalI=[0, 11, 8], S=123456.789, A=9.999999995e+5,
         I=1.0e-300, ilevelF=999998, ilevelI=999997, ndegF=2, ndegI=1,
         t=[5.0000000005e-1, 0, 2.4999999995e-1, 0]),
    # no classes, no modes, zeros
    dict(jF=0, jI=1, symF="A1", symI="B2", eF=0.0, eI=0.0, nu=0.0, cgF=["A1"], cgI=["B2"],
         krotF=0, krotI=1, quantaF=[0], quantaI=[0], normalF=[0], normalI=[0], S=0.0, A=0.0,
         I=0.0, ilevelF=0, ilevelI=0, ndegF=1, ndegI=2, t=[0.0, -0.0, 0, 0]),
]


def printf_sequence(ref_dir):
    src = open(os.path.join(ref_dir, "cuda_host.cu")).read()
    start = src.index("#pragma omp critical(output_ls)")
    end = src.index('printf("\\n");', start) + len('printf("\\n");')
    fmts = []
    for line in src[start:end].splitlines():
        if line.strip().startswith("//"):
            continue
        for m in re.finditer(r'printf\("((?:[^"\\]|\\.)*)"', line):
            fmts.append(m.group(1).encode().decode("unicode_escape"))
    convs = [" ".join(re.findall(r"%[-0-9.]*[a-z]", f)) for f in fmts]
    assert convs == EXPECT, convs
    return fmts


def main():
    ref_dir = os.environ.get("REF_DIR")
    if not ref_dir or not os.path.isfile(os.path.join(ref_dir, "cuda_host.cu")):
        sys.exit("set REF_DIR to the reference checkout")
    subprocess.check_call(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")],
                          env=dict(os.environ, REF_DIR=ref_dir))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref.so"))
    branch = ref._Z6branchii  # const char* branch(int jF, int jI)
    branch.restype = C.c_char_p
    libc = C.CDLL(None)
    fm = printf_sequence(ref_dir)
    buf = C.create_string_buffer(4096)

    def pf(fmt, *args):
        conv = []
        for a in args:
            if isinstance(a, float):
                conv.append(C.c_double(a))
            elif isinstance(a, int):
                conv.append(C.c_int(a))
            else:
                conv.append(C.c_char_p(a.encode()))
        n = libc.snprintf(buf, len(buf), fmt.encode(), *conv)
        assert 0 <= n < len(buf)
        return buf.value.decode()

    out = []
    for f in CASES:
        nclasses, nmodes = len(f["cgF"]) - 1, len(f["quantaF"]) - 1
        s = pf(fm[0], f["jF"], f["symF"], f["jI"], f["symI"],
               branch(f["jF"], f["jI"]).decode(), f["eF"], f["eI"], abs(f["nu"]), f["cgF"][0],
               f["krotF"])
        for i in range(1, nclasses + 1):
            s += pf(fm[1], f["cgF"][i])
        s += pf(fm[2])
        for i in range(1, nmodes + 1):
            s += pf(fm[3], f["quantaF"][i])
        s += pf(fm[4], f["cgI"][0], f["krotI"])
        for i in range(1, nclasses + 1):
            s += pf(fm[5], f["cgI"][i])
        s += pf(fm[6])
        for i in range(1, nmodes + 1):
            s += pf(fm[7], f["quantaI"][i])
        s += pf(fm[8], f["S"], f["A"], f["I"], f["ilevelF"] + 1, f["ilevelI"] + 1, 0, 0)
        for i in range(1, nmodes + 1):
            s += pf(fm[9], f["normalF"][i])
        s += pf(fm[10])
        for i in range(1, nmodes + 1):
            s += pf(fm[11], f["normalI"][i])
        s += pf(fm[12])
        for dF in range(f["ndegF"]):
            for dI in range(f["ndegI"]):
                s += pf(fm[13], f["t"][dI + 2 * dF])
        s += pf(fm[14])
        out.append(dict(fields=f, text=s))
    with open(os.path.join(HERE, "line_format_ref.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print(f"wrote {len(out)} lines")


if __name__ == "__main__":
    main()
