"""Regenerates the golden fixtures in this folder from the ElVibRot source tree.

Run once in a checkout that has the reference mounted (default path below, or
pass it as argv[1]); the fixtures are committed so the tests never need the
reference at run time.

  hermquadra.json : Internal_data/HermQuadra/herm{1..40}.txt -- Gauss-Hermite
                    nodes (column 2), weights (column 3) and weights*exp(x^2)
                    (column 4), parsed to IEEE doubles.
  hh_levels.json  : Working_tests/MPI_tests/{6D,21D}_Davidson_S0/benchmark --
                    the lowest Henon-Heiles SG4 levels (hartree) with the run
                    parameters read from the matching shell_run/run_jobs
                    (6-D: L=LB=LG=3, L_TO_nq B=2; 21-D: L=2, B=2; lambda from
                    sub_system_HenonHeiles.f).
"""
import json
import os
import re
import sys

ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
here = os.path.dirname(os.path.abspath(__file__))

herm = {}
for nq in range(1, 41):
    rows = [l.split() for l in open(os.path.join(ref, "Internal_data/HermQuadra", f"herm{nq}.txt")) if l.strip()]
    herm[str(nq)] = {"x": [float(r[1]) for r in rows], "w": [float(r[2]) for r in rows],
                     "wrho": [float(r[3]) for r in rows]}
json.dump({"source": "Internal_data/HermQuadra/herm{nq}.txt", "nq": herm},
          open(os.path.join(here, "hermquadra.json"), "w"), indent=0)

levels = {}
for name, D in (("6D_Davidson_S0", 6), ("21D_Davidson_S0", 21)):
    d = os.path.join(ref, "Working_tests/MPI_tests", name)
    bench = [float(l.split()[0]) for l in open(os.path.join(d, "benchmark")) if l.strip()]
    jobs = open(os.path.join(d, "run_jobs")).read().strip().splitlines()[-1].split()
    pot = open(os.path.join(d, "sub_system_HenonHeiles.f")).read()
    lam = float(re.search(r"lambda\s*=\s*([0-9.]+)d0", pot).group(1))
    if D == 6:
        L, B = int(jobs[2]), 2          # ./shell_run cores L dav ; B fixed in shell_run
    else:
        L, B = int(jobs[2]), int(jobs[3])   # ./shell_run cores L B dav
    levels[name] = {"D": D, "L": L, "LB": L, "L_TO_nq_A": 1, "L_TO_nq_B": B, "lambda": lam,
                    "Type_HamilOp": 1, "G": "identity (Cartesian, mass 1)",
                    "levels_au": bench,
                    "davidson_conv_resi_au": 0.0005}
json.dump({"source": "Working_tests/MPI_tests/*/benchmark", "cases": levels},
          open(os.path.join(here, "hh_levels.json"), "w"), indent=1)
print("ok")
