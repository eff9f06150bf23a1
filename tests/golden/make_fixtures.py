"""Copy the reference's regression gold vectors used to pin the oracle.

Sources in phoebus's tst/regression/:
- linear_modes.gold: 1638 values, p.density then p.velocity components of
  the final state of the 64^2 linear-modes run, every 10th value, compared
  with soft_equiv at tol 1e-3;
- bondi.gold: 512 values, p.density then p.velocity components of the final
  state (t = 100) of the 128-zone FMKS Bondi run, every value, tol 1e-5.
Run from the repo
root with the reference mounted; the copy is committed so the tests do not
need the reference at run time.
"""
import shutil
import sys
from pathlib import Path

REF = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
HERE = Path(__file__).resolve().parent
for name in ("linear_modes.gold", "bondi.gold"):
    shutil.copyfile(REF / "tst" / "regression" / name, HERE / name)
    print("copied", name)
