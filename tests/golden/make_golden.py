"""Extract the reference's own golden scalars for the compact-operator path.

Reads the reference test-case files as text (they are Python fragments that
``tests/run_tests.py`` executes) and writes ``reference_scalars.json``; copies
the reference's profile baselines of the 2-D Euler, cylindrical and
spherical Sod, Kelvin-Helmholtz and curvilinear O-mesh cases
(``tests/baselines/*.dat``: two rows, x and the profile, compared by
``tests/testObj.py:checkProfile``) next to it.  Run it where the reference
tree is mounted, naming its root:

    python tests/golden/make_golden.py /path/to/pyranda
"""
import json
import os
import shutil
import sys

CASES = {
    "test1DAdvection.py": ["advec-1d-50", "advec-1d-100", "advec-1d-200", "advec-1d-300", "advec-1d-400"],
    "testUnit.py": ["unit-test-3D"],
    "testTaylorGreen.py": ["taylorgreen"],
    "testShuOsher.py": ["shu-osher-CR"],
    "testHeat1D.py": ["heat1D-analytic-16", "heat1D-analytic-32", "heat1D-analytic-64", "heat1D-analytic-128",
                      "heat1D-analytic-256"],
    "testIntegration.py": ["integration-25", "integration-50", "integration-100", "integration-200",
                           "integration-400"],
}


PROFILES = {  # test name -> baseline file (tests/cases/test2deuler.py:3-9)
    "euler-2d-64": "euler-2d-64.dat",
    "euler-2d-128": "euler-2d-128.dat",
    "KH-2d-64": "KelvinHelmholtzKH-2d-64.dat",
    "euler-RZ-128": "euler-RZ-128.dat",
    "euler-SPH-1D": "euler-SPH-1D.dat",
    "euler-SPH-2D": "euler-SPH-2D.dat",
    "cylinder_omesh-2d-64": "cylinder_omesh-2d-64.dat",  # tests/cases/testCylinder.py:33-37
}


def main(root):
    out = {"source": "pyranda tests/cases (baselines blocks)", "tolerance_rel": 1.0e-4, "values": {}}
    for fname, names in CASES.items():
        path = os.path.join(root, "tests", "cases", fname)
        text = open(path).read()
        block = text.split('baselines = """')[1].split('"""')[0]
        for line in block.split("\n"):
            if "--" not in line:
                continue
            name, val = [s.strip() for s in line.split("--")[:2]]
            if name in names:
                out["values"][name] = {"value": float(val), "file": "tests/cases/" + fname}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_scalars.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", dst)
    here = os.path.dirname(dst)
    for name, fname in PROFILES.items():
        shutil.copyfile(os.path.join(root, "tests", "baselines", fname), os.path.join(here, fname))
        print("copied", fname, "for", name)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of the pyranda source tree>")
    main(sys.argv[1])
