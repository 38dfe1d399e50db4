"""Generates tests/golden/ceos_agc.npz: the receiver-attenuation codes of the
96 range lines held by tests/golden/wk_cd_crop.npz (lines 1500..1595 of the
reference's extracted RADARSAT-1 scene, which starts at file line 7769:
code/data_process/CEOS/specify_parameters.m, CD_run_params.mat), taken from
the reference's code/data_process/CEOS/AGC_attenuation_values.mat.  Run where
the reference tree exists:

    python tests/golden/gen_ceos_golden.py <reference checkout>
"""
import os
import sys

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root: str):
    d = os.path.join(ref_root, "code", "data_process", "CEOS")
    agc = sio.loadmat(os.path.join(d, "AGC_attenuation_values.mat"))["nom_attenuation"].ravel()
    p = sio.loadmat(os.path.join(d, "CD_run_params.mat"))
    first_line = int(p["first_rg_line"][0, 0])   # 1-based file line of the scene's first line
    first_cell = int(p["first_rg_cell"][0, 0])   # 1-based range cell of the scene's first cell
    lines = np.arange(1500, 1596) + first_line - 1
    np.savez_compressed(os.path.join(HERE, "ceos_agc.npz"), agc_db=agc[lines].astype(np.int16),
                        scene_first_line=first_line, scene_first_cell=first_cell)
    print("agc", np.unique(agc[lines]), "first line", first_line, "first cell", first_cell)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SARBP_REFERENCE_DIR")
    if not src:
        sys.exit(f"usage: {sys.argv[0]} <reference checkout> (or set SARBP_REFERENCE_DIR)")
    main(src)
