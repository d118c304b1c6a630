"""Generate the golden fixtures in this folder.

  kat_4x6.json      the reference's own known-answer test, read from its test
                    source: test/src/test_shared_loop.cpp:15-34 (same fixture in
                    test_naive.cpp, test_shared_sync.cpp, test_shared_opt.cpp,
                    test_distributed_loop.cpp).  Input rows [1,2,3,4,pad,pad],
                    expected output row 0 = (40,0), (-8,8), (-8,0), rest 0.
  rfft2_small.npz   seeded random inputs with numpy.fft.rfft2 (pocketfft, an
                    FFT implementation independent of the oracle) outputs.

The reference itself cannot run here (HPX and FFTW are absent), so these are
the pins: its KAT, an independent FP64 FFT, and the closed forms the tests
derive (ramp input of examples/hpxfft/shared_loop_2d.cpp:33-40).

Run:  python tests/golden/make_golden.py
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

SHAPES = [(4, 4), (1, 2), (2, 6), (3, 10), (8, 8), (6, 12), (16, 30), (20, 24), (32, 64), (15, 40), (48, 96), (64, 128)]


def main():
    kat = {
        "source": "test/src/test_shared_loop.cpp:15-34",
        "n_row": 4,
        "n_col": 6,
        "input_rows": [[1.0, 2.0, 3.0, 4.0, 0.0, 0.0]] * 4,
        "expected": [[40.0, 0.0, -8.0, 8.0, -8.0, 0.0], [0.0] * 6, [0.0] * 6, [0.0] * 6],
    }
    with open(os.path.join(HERE, "kat_4x6.json"), "w") as f:
        json.dump(kat, f, indent=1)

    rng = np.random.default_rng(20241203)
    arrays = {}
    for nx, ny in SHAPES:
        x = rng.uniform(0.0, 1.0, size=(nx, ny))
        arrays[f"x_{nx}x{ny}"] = x
        arrays[f"X_{nx}x{ny}"] = np.fft.rfft2(x)
    np.savez_compressed(os.path.join(HERE, "rfft2_small.npz"), **arrays)


if __name__ == "__main__":
    main()
