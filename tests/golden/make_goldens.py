"""Extract the reference's blessed outputs into tests/golden/reference_goldens.json.

Reads the serial/parallel `*.output` files of the reference's own regression
tests (tests/solid/<case>/<case>_serial.output, tests/heat/<case>/*.output of
davidscn/matrix-free-dealii-precice) and records the pinned numbers: Newton
iterations per time step, the watchpoint displacement after each step, the
average CG iteration count, and the heat L2 errors.  Run once in a checkout
that has the reference; the JSON it writes is committed and is what the tests
read (the reference tree is not needed at test time).

    python tests/golden/make_goldens.py /path/to/reference
"""
import glob
import json
import os
import re
import sys


def parse_solid(path):
    txt = open(path).read()
    newton = [int(x) for x in re.findall(r"Converged in (\d+) Newton", txt)]
    disp = [[float(a), float(b)] for a, b in
            re.findall(r"displacement: (\S+) (\S+)", txt)]
    avg = int(re.search(r"Average CG iter = (\d+)", txt).group(1))
    dofs = int(re.search(r"Number of degrees of freedom: (\d+)", txt).group(1))
    cells = int(re.search(r"Number of active cells: (\d+)", txt).group(1))
    vol = float(re.search(r"Reference volume: (\S+)", txt).group(1))
    return dict(newton_its=newton, watch_disp=disp, avg_cg=avg, n_dofs=dofs,
                n_cells=cells, ref_volume=vol)


def parse_prm(path):
    out = {}
    for line in open(path):
        m = re.match(r"\s*set\s+(.+?)\s*=\s*(.+?)\s*$", line)
        if m:
            out[m.group(1)] = m.group(2)
    return out


def main(ref):
    goldens = {"source": "davidscn/matrix-free-dealii-precice tests/", "solid": {}, "heat": {}}
    for d in sorted(glob.glob(os.path.join(ref, "tests", "solid", "*"))):
        name = os.path.basename(d)
        ser = os.path.join(d, name + "_serial.output")
        if not os.path.exists(ser):
            continue
        entry = parse_solid(ser)
        par = os.path.join(d, name + "_parallel.output")
        entry["parallel_identical"] = os.path.exists(par) and parse_solid(par) == entry
        prm = parse_prm(os.path.join(d, name + ".prm"))
        entry["prm"] = {k: prm[k] for k in ("MF caching", "Preconditioner type",
                                            "Formulation", "Polynomial degree",
                                            "Quadrature order", "Global refinement",
                                            "Time step size", "End time") if k in prm}
        goldens["solid"][name] = entry
    for d in sorted(glob.glob(os.path.join(ref, "tests", "heat", "*"))):
        if not os.path.isdir(d):
            continue
        name = os.path.basename(d)
        ser = os.path.join(d, name + "_serial.output")
        if not os.path.exists(ser):
            continue
        errs = [float(x) for x in re.findall(r"Error: (\S+)", open(ser).read())]
        goldens["heat"][name] = {"l2_errors": errs, "max_l2_error": max(errs)}
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")
    with open(out, "w") as f:
        json.dump(goldens, f, indent=1, sort_keys=True)
    print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_goldens.py <path of the reference checkout>")
    main(sys.argv[1])
