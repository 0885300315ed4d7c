#!/usr/bin/env python3
"""Extracts member function definitions of FEDDLib's FE class template from
feddlib/core/FE/FE_def.hpp (test infrastructure only).

FE_def.hpp does not compile outside a Trilinos build (it includes Thyra /
Xpetra headers and the un-vendored aceinterface.hpp), so the checker takes
the few member functions it needs out of the reference file as they are and
compiles them against this project's stub FE class (oracle/ref_fe_stub.hpp).
The output goes to oracle/_ref/ only and is never committed.

    python3 oracle/extract_fe_members.py <FEDDLib tree> <output .inc>
"""
import re
import sys

# (name, a fragment of its parameter list that selects the overload)
MEMBERS = [
    ("nh3d", "double* v"),
    ("epsilonTensor", "vec_dbl_Type &basisValues"),
    ("applyBTinv", "SmallMatrix<SC>& Binv"),
    ("buildFullDPhi", "vec3D_dbl_ptr_Type dPhi"),
    ("fillMatrixArray", "SmallMatrix<double> &matIn"),
    ("assemblyLinElasXDim", "double lambda"),
    ("assemblyElasticityJacobianAceFEM", "MatrixPtr_Type &A"),
    ("assemblyElasticityStressesAceFEM", "MultiVectorPtr_Type &f"),
    ("assemblyRHS", "RhsFunc_Type func"),
]


def body_end(src, start):
    """Index just past the brace that closes the first '{' at or after start
    (comments and string literals skipped)."""
    i, depth, n = src.index("{", start), 0, len(src)
    while i < n:
        c = src[i]
        if src.startswith("//", i):
            i = src.index("\n", i)
            continue
        if src.startswith("/*", i):
            i = src.index("*/", i) + 2
            continue
        if c == '"':
            i += 1
            while src[i] != '"':
                i += 2 if src[i] == "\\" else 1
        elif c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced braces")


def extract(src, name, selector):
    pat = re.compile(r"template\s*<class SC, class LO, class GO, class NO>\s*\n\s*void\s+FE<SC,LO,GO,NO>::"
                     + name + r"\s*\(")
    for m in pat.finditer(src):
        head_end = src.index("{", m.end())
        if selector in src[m.end():head_end]:
            return src[m.start():body_end(src, m.start())]
    raise KeyError(f"FE::{name} ({selector}) not found")


def main():
    tree, out = sys.argv[1], sys.argv[2]
    src = open(f"{tree}/feddlib/core/FE/FE_def.hpp").read()
    parts = [f"// extracted from feddlib/core/FE/FE_def.hpp: FE::{n}\n" + extract(src, n, s) for n, s in MEMBERS]
    with open(out, "w") as f:
        f.write("\n\n".join(parts) + "\n")


if __name__ == "__main__":
    main()
