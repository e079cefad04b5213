"""Write tests/golden/fdm_coeffs.json from the reference's own coefficient script,
Utils/FDMcoeffs.py: the flux-form face coefficients of the 8-point first-derivative stencil
from -4 (UP7 of run.jl:75) and of the 7-point one from -3 (CD6 of run.jl:76, with its leading
zero), and the half-and-half blend the script prints. Runs where the reference is present:

  python tests/golden/make_fdm_coeffs.py <root of the reference source tree>
"""
import argparse
import json
import runpy
from pathlib import Path

import numpy as np

ap = argparse.ArgumentParser()
ap.add_argument("ref", help="root of the reference source tree")
ref = Path(ap.parse_args().ref)
ns = runpy.run_path(str(ref / "Utils" / "FDMcoeffs.py"))  # the script prints its blend
up7 = ns["fluxCoeff"](8, -4)
cd6 = np.concatenate(([0.0], ns["fluxCoeff"](7, -3)))
out = {"source": "Utils/FDMcoeffs.py fluxCoeff(8, -4), fluxCoeff(7, -3)",
       "up7": up7.tolist(), "cd6": cd6.tolist(), "blend_half": (0.5 * up7 + 0.5 * cd6).tolist()}
path = Path(__file__).resolve().parent / "fdm_coeffs.json"
path.write_text(json.dumps(out, indent=1) + "\n")
print(path)
