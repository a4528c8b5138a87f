"""ORACLE BUILD SUPPORT (test infrastructure only).

The reference translation units compiled for oracle/_ref/ name many functions of the reference library that
a single-process run of the level-set path never reaches (Poisson solvers, MLS quadrature, refinement
criteria, ...). This script lists the symbols a trial link leaves undefined and writes a C file that defines
each of them as a function that reports its name and aborts, so the final link can require every symbol to
be resolved. A run that does reach one of them stops with that name instead of returning a wrong answer.

usage: python3 ref_autostubs.py <trial .so> <out .c>
"""
import subprocess
import sys


def undefined_symbols(lib):
    out = subprocess.run(["nm", "-D", "--undefined-only", lib], check=True, stdout=subprocess.PIPE, text=True).stdout
    names = []
    for line in out.splitlines():
        parts = line.split()
        if len(parts) != 2:
            continue
        kind, name = parts
        if kind != "U" or "@" in name:  # weak or versioned (C and C++ run-time libraries)
            continue
        names.append(name)
    return sorted(set(names))


def main():
    lib, out = sys.argv[1], sys.argv[2]
    names = undefined_symbols(lib)
    with open(out, "w") as fh:
        fh.write("/* generated by ref_autostubs.py: symbols the single-process reference build does not provide */\n")
        fh.write("#include <stdio.h>\n#include <stdlib.h>\n")
        fh.write("static void ref_unreached(const char *s) {\n"
                 "  fprintf(stderr, \"reference build: %s is outside this single-process build\\n\", s);\n  abort();\n}\n")
        for i, n in enumerate(names):
            fh.write(f"void ref_stub_{i}(void) __asm__(\"{n}\");\n")
            fh.write(f"void ref_stub_{i}(void) {{ ref_unreached(\"{n}\"); }}\n")
    print(f"{len(names)} symbols stubbed -> {out}")


if __name__ == "__main__":
    main()
