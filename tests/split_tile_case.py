"""Runs one split-precision MFT case in a fresh process (the tile override is read once per process).

Prints the relative L2 errors of forward, backward and adjoint against the float64 oracle, one per line.
Used by test_split_gpu.test_split_tile_configurations with HX_SPLIT_TILE set.
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import numpy as np  # noqa: E402

import hcipy_gb300 as hg  # noqa: E402
from oracle import fourier as ofourier  # noqa: E402


def main():
    rng = np.random.default_rng(11)
    n_in, n_out = 200, 150
    xg = (np.arange(n_in) - n_in / 2 + 0.5) / n_in
    ug = (np.arange(n_out) - n_out / 2 + 0.5) * 0.37
    gi = hg.CartesianGrid(hg.SeparatedCoords([xg, xg]))
    go = hg.CartesianGrid(hg.SeparatedCoords([ug, ug]))
    mft = hg.MatrixFourierTransform(gi, go, precision='split')
    e = (rng.standard_normal((2, gi.size)) + 1j * rng.standard_normal((2, gi.size))).astype(np.complex64)
    f = (rng.standard_normal((2, go.size)) + 1j * rng.standard_normal((2, go.size))).astype(np.complex64)
    fw, bw, ad = mft.forward(e).numpy(), mft.backward(f).numpy(), mft.adjoint(f).numpy()
    errs = []
    for i in range(2):
        for got, ref in ((fw[i], ofourier.mft_forward(e[i].astype(complex), xg, xg, ug, ug, gi.weights)),
                         (bw[i], ofourier.mft_backward(f[i].astype(complex), xg, xg, ug, ug, go.weights)),
                         (ad[i], ofourier.mft_adjoint(f[i].astype(complex), xg, xg, ug, ug, gi.weights))):
            errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    import torch
    status = mft._plan(torch.complex64).status()
    print(' '.join('%.3e' % x for x in errs), status)


if __name__ == '__main__':
    main()
