"""Extracts the known-answer CSR systems of the reference's CSRMatrixGeneratorTest.cpp into
csr_generator_test.json (row pointers, columns, values and right-hand sides of
`1.0 == d2x(e) + d2y(e)` on a 4x4-cell grid with h = 1 for Dirichlet, Neumann and periodic
boundaries; the Neumann and periodic systems pin the last row).  Reads the test file as text.

    python tests/golden/extract_csr_golden.py [path/to/OpFlow]    (default: $OPFLOW_REFERENCE)
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OPFLOW_REFERENCE")
    if not ref:
        sys.exit("name the OpFlow source tree (argument or $OPFLOW_REFERENCE)")
    src = open(os.path.join(ref, "test/Core/Equation/CSRMatrixGeneratorTest.cpp")).read()
    out = {}
    for name, bc in (("SimplePoisson", "dirc"), ("SimplePoisson_Neum", "neum"), ("SimplePoisson_Periodic", "periodic")):
        m = re.search(r"TEST_F\(CSRMatrixGeneratorTest, %s\)\s*\{(.*?)\n\}" % re.escape(name), src, re.S)
        body = m.group(1)
        arrs = {}
        for key in ("ptr", "col", "val", "rhs"):
            mm = re.search(r"\b%s\s*\{([^}]*)\}" % key, body)
            arrs[key] = [float(v) if key in ("val", "rhs") else int(v) for v in mm.group(1).replace("\n", " ").split(",")]
        pin = "generate<0>(st, DS::ColoredMDRangeMapper<2> {p.assignableRange}, true)" in body
        out[bc] = dict(arrs, pin_last_row=pin, source="test/Core/Equation/CSRMatrixGeneratorTest.cpp:%s" % name)
    json.dump(out, open(os.path.join(HERE, "csr_generator_test.json"), "w"), indent=1)
    print({k: len(v["val"]) for k, v in out.items()})


if __name__ == "__main__":
    main()
