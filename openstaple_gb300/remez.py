"""Command-line generator of .REMEZ files, with the arguments of the
reference's offline program (RationalApprox/rationalapprox_calc.cc:20-95):

    python -m openstaple_gb300.remez tolerance exponent_num exponent_den lambda_min [order]

It computes the approximation with the library's generator
(ostaple_remez_generate: the order guessed as the reference does, or the
given one, raised until the error is at most the tolerance) and writes it
under the reference's file name (rational_approx_filename) with the
library's rationalapprox_save, in the current directory.  Host code only: no
GPU is used."""
from __future__ import annotations

import ctypes as C
import sys


def main(argv: list[str]) -> int:
    if len(argv) not in (4, 5):
        print("Use as arguments:    tolerance exponent_num exponent_den lambda_min (optional: min approx order)")
        return 0
    from . import api
    from .native import lib
    goal, num, den, lmin = float(argv[0]), int(argv[1]), int(argv[2]), float(argv[3])
    order = int(argv[4]) if len(argv) == 5 else 0
    ra = api.remez(num, den, lmin, order=order, goal_error=goal)
    L = lib()
    name = C.string_at(L.rational_approx_filename(goal, num, den, lmin))
    L.rationalapprox_save(name, C.byref(ra))
    print(f"f(x) = (x)^({num}/{den}) on [{lmin:e}, 1]: order {ra.approx_order}, error {ra.error:e}")
    print(f"Written file {name.decode()} .")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
