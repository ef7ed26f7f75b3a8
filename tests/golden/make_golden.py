"""Copy the reference's golden vectors for the smoother path into ``tests/golden/``.

Run once with the path of a checkout of the reference as the argument
(``python make_golden.py <reference checkout>``); the outputs are committed so
the tests never read the reference at run time.

* ``bearings_ys.npy``, ``ieks.npz``, ``icks.npz`` - observations and the
  100-iteration extended and cubature smoother outputs of the bearings
  regression test (tests/test_bearings_only.py:25-72 of the reference).
* ``robustness_small.npz`` - the first 100 observations of runs 1..20 of
  ``notebooks/robustness_data/data-T8000-Run*.npz`` and the FP32 GPU
  log-likelihoods the reference computed on them for T in 20..100
  (notebooks/robustness_100runs.py:46-69 and the saved
  ``ell_float32_{cubature,extended}_{sqrt,std}_100runs.npz``: square-root and
  covariance form; NaN where the reference's FP32 run failed).
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(REF):
    shutil.copyfile(f"{REF}/tests/bearings/ys.npy", f"{HERE}/bearings_ys.npy")
    with np.load(f"{REF}/tests/bearings/ieks.npz") as d:
        np.savez_compressed(f"{HERE}/ieks.npz", mean=d["arr_0"], cov=d["arr_1"])
    with np.load(f"{REF}/tests/bearings/icks.npz") as d:
        np.savez_compressed(f"{HERE}/icks.npz", mean=d["arr_0"], cov=d["arr_1"])
    base = f"{REF}/notebooks/robustness_data"
    runs = 20
    ys = np.stack([np.load(f"{base}/data-T8000-Run{j + 1}.npz")["data"][:100] for j in range(runs)])
    Ts = np.array([20, 30, 40, 50, 80, 100])
    with np.load(f"{base}/ell_float32_cubature_sqrt_100runs.npz") as d:
        ell_cub = d["gpu_ICKS_sqrt_par_ell"][:len(Ts), :runs]
    with np.load(f"{base}/ell_float32_extended_sqrt_100runs.npz") as d:
        ell_ext = d["rts_gpu_IEKS_sqrt_par_ell"][:len(Ts), :runs]
    with np.load(f"{base}/ell_float32_cubature_std_100runs.npz") as d:
        ell_cub_std = d["gpu_ICKS_std_par_ell"][:len(Ts), :runs]
    with np.load(f"{base}/ell_float32_extended_std_100runs.npz") as d:
        ell_ext_std = d["rts_gpu_IEKS_std_par_ell"][:len(Ts), :runs]
    np.savez_compressed(f"{HERE}/robustness_small.npz", ys=ys, Ts=Ts, ell_cubature=ell_cub,
                        ell_extended=ell_ext, ell_cubature_std=ell_cub_std, ell_extended_std=ell_ext_std)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout>")
    main(sys.argv[1])
