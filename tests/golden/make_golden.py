"""Regenerates the golden fixtures in this folder from the ElVibRot source tree.

Run once with the path of an ElVibRot checkout as the only argument
(python make_golden.py <ElVibRot source tree>); the fixtures are committed so
the tests never need the reference at run time.

  hermquadra.json : Internal_data/HermQuadra/herm{1..40}.txt -- Gauss-Hermite
                    nodes (column 2), weights (column 3) and weights*exp(x^2)
                    (column 4), parsed to IEEE doubles.
  hh_levels.json  : Working_tests/MPI_tests/{6D,21D}_Davidson_S0/benchmark --
                    the lowest Henon-Heiles SG4 levels (hartree) with the run
                    parameters read from the matching shell_run/run_jobs
                    (6-D: L=LB=LG=3, L_TO_nq B=2; 21-D: L=2, B=2; lambda from
                    sub_system_HenonHeiles.f).
  pyrazine12d.json: Working_tests/MPI_tests/12D_propagation_S0 -- the
                    61-row autocorrelation <psi0|psi(t)> of the 2-state, 12-mode
                    pyrazine SG4 propagation (benchmark), with the run
                    parameters from shell_run/run_jobs, the model constants
                    parsed from sub_system_pyrazine.f and calc_f2_f1Q.f90, and
                    the eV->hartree factor recomputed from the CODATA 2006
                    constants of Ext_Lib/ConstPhys_loc/SRC/sub_module_constant.f90
                    (the reference's default version) with its formulas.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2 or not os.path.isdir(sys.argv[1]):
    sys.exit("usage: python make_golden.py <path of the ElVibRot source tree>")
ref = sys.argv[1]
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

# --- 2-state pyrazine propagation -------------------------------------------
import math

d = os.path.join(ref, "Working_tests/MPI_tests/12D_propagation_S0")
num = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eEdD][-+]?\d+)?"


def fortran_array(text, name):
    """Values of `name(ndim) = (/ ... /)` or `[ ... ]` (ZERO -> 0)."""
    m = re.search(name + r"\(ndim\)\s*=\s*(?:\(/|\[)(.*?)(?:/\)|\])", text, re.S)
    body = re.sub(r"\n\s*\*", " ", m.group(1)).replace("&", " ")
    vals = []
    for tok in body.split(","):
        tok = tok.strip()
        if tok.upper() == "ZERO":
            vals.append(0.0)
        elif tok:
            vals.append(float(re.match(num, tok).group(0).replace("d", "e").replace("D", "e")))
    return vals


pot = open(os.path.join(d, "sub_system_pyrazine.f")).read()
keo = open(os.path.join(d, "calc_f2_f1Q.f90")).read()
w, k1, k2 = fortran_array(pot, "w"), fortran_array(pot, "k1"), fortran_array(pot, "k2")
assert fortran_array(keo, "w") == w and len(w) == 12
delta = float(re.search(r"delta\s*=\s*(" + num + ")_Rkind", pot).group(1))
lam = float(re.search(r"lambda\s*=\s*(" + num + ")_Rkind", pot).group(1))
const = open(os.path.join(ref, "Ext_Lib/ConstPhys_loc/SRC/sub_module_constant.f90")).read()
i0 = const.index("SUBROUTINE constantes_CODATA2006")
blk = const[i0:const.index("END SUBROUTINE constantes_CODATA2006")]
cv = {k: float(re.search(r"\n\s*" + k + r"\s*=\s*(" + num + ")_Rkind", blk).group(1)) for k in ("c", "h", "e", "me")}
# the reference's formulas (sub_constantes): mhu0 = pi*4e-7, epsi0 = 1/(mhu0 c^2),
# hb = h/(2 pi), a0 = (hb/e)^2/me*4*pi*epsi0, Eh = (e e/a0)/(4 pi epsi0), auTOeV = Eh/e;
# the 'eV' unit stores 1/auTOeV and get_Conv_au_TO_unit returns its inverse.
pi = math.pi
mhu0 = pi * 4.0e-7
epsi0 = 1.0 / (mhu0 * cv["c"] * cv["c"])
hb = cv["h"] / (2.0 * pi)
a0 = (hb / cv["e"]) ** 2 / cv["me"] * 4.0 * pi * epsi0
Eh = (cv["e"] * cv["e"] / a0) / (4.0 * pi * epsi0)
auTOeV = Eh / cv["e"]
eVTOau = 1.0 / (1.0 / (1.0 / auTOeV))
shell = open(os.path.join(d, "shell_run")).read()
Bs = {k: int(re.search(r"\n" + k + r"=(\d+)", shell).group(1)) for k in ("B1", "B2", "B3", "B4", "B")}
jobs = open(os.path.join(d, "run_jobs")).read().strip().splitlines()[-1].split()   # ./shell_run cores L
L = int(jobs[2])
wp0 = re.search(r"\n\s*((?:\d+\s+){14})(" + num + r")\s+(" + num + r")\s*\n", shell)
idx = [int(v) for v in wp0.group(1).split()]
rows = [[float(v) for v in line.split()] for line in open(os.path.join(d, "benchmark")) if line.strip()]
json.dump({"source": "Working_tests/MPI_tests/12D_propagation_S0 (benchmark, shell_run, run_jobs, "
                     "sub_system_pyrazine.f, calc_f2_f1Q.f90); CODATA2006 in sub_module_constant.f90",
           "D": 12, "L": L, "LB": L, "nb0": 2,
           "L_TO_nq_A": [1] * 12, "L_TO_nq_B": [Bs["B1"], Bs["B2"], Bs["B3"], Bs["B4"]] + [Bs["B"]] * 8,
           "basis": "Hm, Q0=0, scaleQ=1, nb(l)=nq(l)",
           "omega_eV": w, "kappa1_eV": k1, "kappa2_eV": k2, "delta_eV": delta, "lambda_eV": lam,
           "codata2006": cv, "eV_to_hartree": eVTOau,
           "keo": "Tdef2(i,i) = -1/2 omega_i (eV->hartree), f1 = 0 (type 1)",
           "potential": "V11 = 1/2 sum w Q^2 - delta + sum k1 Q, V22 = 1/2 sum w Q^2 + delta + sum k2 Q, "
                        "V12 = V21 = lambda Q_1 (eV->hartree)",
           "psi0": {"nDval": idx[:12], "i_h": idx[12], "i_e": idx[13], "coef": [float(wp0.group(2)),
                                                                                 float(wp0.group(3))]},
           "propagation": "Chebyshev (type_WPpropa=1), poly_tol=1e-10, npoly<=300",
           "autocorr": {"t_au": [r[0] for r in rows], "re": [r[1] for r in rows], "im": [r[2] for r in rows],
                        "abs": [r[3] for r in rows]},
           "criterion": 1e-8},
          open(os.path.join(here, "pyrazine12d.json"), "w"), indent=1)
print("ok")
