"""Regenerates tests/golden/analysis/: outputs of the reference's own
analysis programs (strain_calc.cpp, axial_contribution.cpp, built unchanged
by oracle/build_ref.sh into oracle/_ref/) on small.dat and the displacement
field of its third shear step in ref_sweep/ (small_3.pos minus the original
points).

Run where the reference checkout exists, after oracle/build_ref.sh:
    python tests/golden/make_analysis_golden.py

Files:
  small_disp.txt     the displacement field (ux uy per node, %.17e)
  ref_strains.txt    strain_calc's output (one strain per bond, %2.10le)
  ref_axial.json     axial_contribution's energy for k = 1 and k = 2.5
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import network_relaxation_gb300 as nr  # noqa: E402


def main():
    ref = os.path.join(ROOT, "oracle", "_ref")
    out = os.path.join(HERE, "analysis")
    os.makedirs(out, exist_ok=True)
    dat = os.path.join(HERE, "small.dat")
    pts = nr.HostNetwork.read(dat).arrays()["points"]
    pos = np.loadtxt(os.path.join(HERE, "ref_sweep", "small_3.pos"))
    disp = pos - pts
    disp_file = os.path.join(out, "small_disp.txt")
    with open(disp_file, "w") as f:
        for ux, uy in disp:
            f.write("%.17e %.17e\n" % (ux, uy))
    subprocess.check_call([os.path.join(ref, "strain_calc"), dat, disp_file, os.path.join(out, "ref_strains.txt")])
    axial = {}
    for k in ("1.0", "2.5"):
        txt = subprocess.check_output([os.path.join(ref, "axial_contribution"), dat, disp_file, k], text=True)
        axial[k] = float(txt.split()[-1])
    with open(os.path.join(out, "ref_axial.json"), "w") as f:
        json.dump(axial, f, indent=1)
    print("analysis fixtures written:", axial)


if __name__ == "__main__":
    main()
