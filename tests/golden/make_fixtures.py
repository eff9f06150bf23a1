"""Copy the reference's regression gold vectors used to pin the oracle.

Sources in phoebus's tst/regression/:
- linear_modes.gold: 1638 values, p.density then p.velocity components of
  the final state of the 64^2 linear-modes run, every 10th value, compared
  with soft_equiv at tol 1e-3;
- bondi.gold: 512 values, p.density then p.velocity components of the final
  state (t = 100) of the 128-zone FMKS Bondi run, every value, tol 1e-5;
- radiation_diffusion.gold: 204 values, r.p.J then r.p.H components of the
  final state (t = 1) of the 512-zone M1 diffusion run (radiation_advection
  pgen, gray scattering tau = 1e3, u^1 = W 0.3), every 10th value, tol 1e-5.
Usage: python tests/golden/make_fixtures.py <phoebus source tree>.  The
copy is committed, so the tests do not need the reference at run time.
"""
import shutil
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: make_fixtures.py <phoebus source tree>")
REF = Path(sys.argv[1])
HERE = Path(__file__).resolve().parent
for name in ("linear_modes.gold", "bondi.gold", "radiation_diffusion.gold"):
    shutil.copyfile(REF / "tst" / "regression" / name, HERE / name)
    print("copied", name)
