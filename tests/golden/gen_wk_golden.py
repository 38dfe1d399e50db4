"""Generates tests/golden/wk_cd_crop.npz from the reference's RADARSAT-1
echo blocks (code/SAR_WK/wk_v5.2.3/data/CDdata1.mat, CDdata2.mat; 3072 x 2048)
with the FP64 omega-K restatement (oracle/wk.py).  Run where the reference
tree exists:

    python tests/golden/gen_wk_golden.py <reference checkout>

Stores:
  echo      a 96 x 64 crop of the echo (rows 1500.., columns 1000..), complex64
  image     its omega-K image (128 x 106), complex64, RADARSAT-1 parameters
  sharp_file, sharp_flip
            normalised sharpness sum|I|^4 / (sum|I|^2)^2 of the full 3072 x 2048
            scene imaged with the parameter file's kr sign and with it flipped
            (pins the sign of the reference function's range term: the file's
            sign focuses the scene)
"""
import os
import sys

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import wk  # noqa: E402


def main(ref_root: str):
    d = os.path.join(ref_root, "code", "SAR_WK", "wk_v5.2.3", "data")
    echo = np.concatenate([sio.loadmat(os.path.join(d, "CDdata1.mat"))["data"],
                           sio.loadmat(os.path.join(d, "CDdata2.mat"))["data"]]).astype(np.complex64)
    p = wk.radarsat1()
    crop = np.ascontiguousarray(echo[1500:1596, 1000:1064])
    img = wk.wk_image(crop.astype(np.complex128), p).astype(np.complex64)
    sharp = {}
    for name, kr in (("file", p.kr), ("flip", -p.kr)):
        q = wk.WkParams(**{**p.__dict__, "kr": kr})
        a2 = np.abs(wk.wk_image(echo.astype(np.complex128), q)) ** 2
        sharp[name] = float(np.sum(a2 * a2) / np.sum(a2) ** 2)
        print(name, "kr", kr, "normalised sharpness", sharp[name])
    np.savez_compressed(os.path.join(HERE, "wk_cd_crop.npz"), echo=crop, image=img,
                        sharp_file=sharp["file"], sharp_flip=sharp["flip"])


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SARBP_REFERENCE_DIR")
    if not src:
        sys.exit(f"usage: {sys.argv[0]} <reference checkout> (or set SARBP_REFERENCE_DIR)")
    main(src)
