"""Extract the golden vectors shipped with the reference's examples into tests/golden/.

Source (reference output files, read as text, run in the build container where the reference is mounted):
  examples/elliptic1d/parabola/run/residual.curve  -- CG residual history (N=5, 10 elements, tol 1e-8)
  examples/elliptic1d/parabola/run/elliptic.curve  -- solution x, u at the GLL nodes
  examples/elliptic1d/parabola/run/runtime.params  -- the namelist that produced them
  examples/shallowwater/dipole/run/Energies.0000000000.curve -- KE and PE of the dipole run at t = 0, 500, 1000
  examples/shallowwater/dipole/run/shallowwater.params      -- the namelist shipped beside it
The fixtures keep the numbers verbatim (residual lines up to the first zero entry after convergence).

    python tests/golden/extract_reference_curves.py /path/to/reference
"""
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/extract_reference_curves.py /path/to/reference")
REF = sys.argv[1]
OUT = os.path.dirname(os.path.abspath(__file__))
run = os.path.join(REF, "examples", "elliptic1d", "parabola", "run")

res = open(os.path.join(run, "residual.curve")).read().splitlines()
keep = []
for line in res:
    keep.append(line)
    parts = line.split()
    if len(parts) == 2 and float(parts[1]) == 0.0:
        break
open(os.path.join(OUT, "elliptic1d_residual.curve"), "w").write("\n".join(keep) + "\n")

sol = open(os.path.join(run, "elliptic.curve")).read().split("#source")[0]
open(os.path.join(OUT, "elliptic1d_solution.curve"), "w").write(sol)
params = open(os.path.join(run, "runtime.params")).read()
open(os.path.join(OUT, "elliptic1d_runtime.params"), "w").write(params)
dip = os.path.join(REF, "examples", "shallowwater", "dipole", "run")
open(os.path.join(OUT, "dipole_energies.curve"), "w").write(open(os.path.join(dip, "Energies.0000000000.curve")).read())
open(os.path.join(OUT, "dipole_shallowwater.params"), "w").write(open(os.path.join(dip, "shallowwater.params")).read())
print("wrote", len(keep), "residual lines and the dipole energy curve")
