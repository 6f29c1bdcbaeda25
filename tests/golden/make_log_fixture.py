"""Extract the reference's logged Newton runs into tests/golden/reference_logs.json.

Source: the reference's Results/<ARM>_<VARIANT>/order<p>-mesh<m>/out-1.txt,
written by its main.cpp (Solution(), main.cpp:160-256) on the meshes
gmsh/wellbore_<m>.msh: the equation count ("Solving a NLS with DOF = "), the
colour count, and per Newton iteration the "delta_du norm" and "residue norm"
lines, up to "Number of iterations = ".  Run from the repository root:

    python tests/golden/make_log_fixture.py [reference_dir]
"""
import json
import os
import re
import sys

# the reference tree: argument, IPFEM_REFERENCE_DIR, or `reference` beside the repository root
REF = sys.argv[1] if len(sys.argv) > 1 else (os.environ.get("IPFEM_REFERENCE_DIR") or os.path.normpath(
     os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference")))
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_logs.json")


def parse(path):
    txt = open(path).read()
    dof = int(re.search(r"DOF = (\d+)", txt).group(1))
    col = re.search(r"Number of colors = (\d+)", txt)
    it = re.search(r"Number of iterations = (\d+)", txt)
    du = [float(x) for x in re.findall(r"delta_du norm = (\S+)", txt)]
    res = [float(x) for x in re.findall(r"Nonlinear process : residue norm = (\S+)", txt)]
    return {"dof": dof, "colors": int(col.group(1)) if col else None, "iterations": int(it.group(1)) if it else None,
            "delta_du": du, "residue": res}


def main():
    out = {"source": "Results/<arm>/order<p>-mesh<m>/out-1.txt of the reference", "runs": {}}
    root = os.path.join(REF, "Results")
    for arm in sorted(os.listdir(root)):
        d = os.path.join(root, arm)
        if not os.path.isdir(d):
            continue
        for case in sorted(os.listdir(d)):
            f = os.path.join(d, case, "out-1.txt")
            if os.path.exists(f):
                run = parse(f)
                if not case.endswith(("-mesh1", "-mesh2")):
                    # meshes 3-5: counts only (the histories replayed are those of meshes 1 and 2)
                    del run["delta_du"], run["residue"]
                out["runs"]["%s/%s" % (arm, case)] = run
    with open(OUT, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print(OUT, len(out["runs"]), "runs")


if __name__ == "__main__":
    main()
