"""Extract the golden values of the reference's own tests for the hot path.

Reads the reference's test/runtests.jl as text (it is not executed) and
writes reference_goldens.json next to this script.  Run it where the
reference is mounted:

    python tests/golden/extract_reference_goldens.py /path/to/reference

The tests covered are the ones on the semi-discrete residual path with
ModalTensor on triangles (test/runtests.jl:38-60 and :111-121).  The 3-D
ModalTensor Tet advection test (:123-129) measures its error with a
Jaskowiec-Sukumar quadrature rule whose node table is not part of the
reference, so its golden cannot be recomputed and is recorded unused.
"""
import json
import os
import re
import sys


def block(text, title):
    start = text.index(f'@testset "{title}"')
    end = text.index("\nend", start)
    return text[start:end]


def floats(s):
    return [float(x) for x in re.findall(r"[-+]?\d+\.\d+(?:e[-+]?\d+)?", s)]


def main(ref_root):
    path = os.path.join(ref_root, "test", "runtests.jl")
    text = open(path).read()
    tol = float(re.search(r"const tol = ([0-9.e-]+)", text).group(1))
    adv = block(text, "Advection 2D Energy-Conservative ModalTensor Tri")
    vortex = block(text, "Isentropic Euler vortex FluxDiff ModalTensor Tri 2D LF")
    tet = block(text, "Advection 3D Energy-Conservative ModalTensor Tet")
    out = {
        "source": "test/runtests.jl",
        "tol": tol,
        "advection_2d_modal_tensor_tri": {
            "lines": "38-60",
            "l2": floats(re.search(r"@test l2 ≈ ([0-9.e-]+)", adv).group(1))[0],
            "conservation": 0.0, "energy": 0.0},
        "euler_vortex_2d_modal_tensor_tri_fd_lf": {
            "lines": "111-121",
            "l2": floats(re.search(r"@test l2 ≈ \[(.*?)\]", vortex, re.S).group(1)),
            "conservation": [0.0, 0.0, 0.0, 0.0]},
        "advection_3d_modal_tensor_tet_unused": {
            "lines": "123-129",
            "l2": floats(re.search(r"@test l2 ≈ ([0-9.e-]+)", tet).group(1))[0],
            "why_unused": "error quadrature JaskowiecSukumarQuadrature(2p+3) table not available"},
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")
    json.dump(out, open(dst, "w"), indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python extract_reference_goldens.py <path to the reference checkout>")
    main(sys.argv[1])
