"""Write tests/golden/drivers_small.npz from the reference's OWN drivers.

Run where the reference sources are present (oracle.reference_dir():
FFTGAL_REFERENCE_DIR, or the checkout oracle/Makefile builds from):

    make -C oracle ref && python tests/golden/make_drivers_golden.py

oracle/Makefile builds src/app/Psb.c, Pss.c, DLsb.c and DLss.c unmodified
against the reference's src/fft.c, gal.c, power.c, io/qpm.c and the shim
FFTW/GSL headers (oracle/_ref/).  This script writes a small synthetic mock in
the QPM cubic text format that src/io/qpm.c reads, runs the four drivers on it
and stores:

  * the catalog as the reference's loader parsed it;
  * Psb / Pss: the Pl and Pmu tables of their first sub-volume (redshift space
    along z, sub-box / sub-sphere 000), and the particles and randoms of that
    sub-volume, reproduced by calling the reference's gal_rsd and the first
    gal_subbox / gal_subsphere of a fresh process, as the driver's first
    iteration does (their random stream starts from the same seed);
  * DLsb / DLss: the DeltaL tables of all six lines of sight.

tests/test_oracle_drivers.py replays the four drivers' computations with the
oracle (oracle/fftgal_oracle.c) and compares.
"""
from __future__ import annotations

import json
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from catalogs import uniform_box  # noqa: E402
from oracle.reflib import available, read_table  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
NG, L, NSUB, ALPHA, DK, A, ID = 16, 100.0, 2, 0.05, 0.08, 0.6, 1
NPART = 2000
LOS6 = [(0, 0, 1), (0, 1, 0), (0, 1, 1), (1, 0, 0), (1, 0, 1), (1, 1, 0)]  # the drivers' loop order

# reproduce the first sub-volume in a fresh process (the reference's static
# random generators start from their seed there, as in the driver)
_FIRST_SUB = r"""
import ctypes as C, json, math, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from oracle.reflib import RefLib
lib = RefLib.lib()
mock, kind, L, Nsub, alpha, a = sys.argv[2], sys.argv[3], float(sys.argv[4]), int(sys.argv[5]), float(sys.argv[6]), float(sys.argv[7])
dp = C.POINTER(C.c_double)
part = lib.gal_loadqpm_cubic(mock.encode(), L)
Om = 0.29
OL = 1 - Om
aH = a * (100 * math.sqrt(Om / (a * a * a) + OL))  # a * H(a) of src/app/Psb.c:14-18
los = np.array([0.0, 0.0, 1.0])
rsd = lib.gal_rsd(part, los.ctypes.data_as(dp), aH)
Lsub = L / Nsub
if kind == "box":
    vol = np.array([0.0, Lsub, 0.0, Lsub, 0.0, Lsub, L])
    sub = lib.gal_subbox(rsd, vol.ctypes.data_as(dp), alpha)
else:
    vol = np.array([0.0, 0.0, 0.0, Lsub * math.sqrt(3) / 2, L])
    sub = lib.gal_subsphere(rsd, vol.ctypes.data_as(dp), alpha)
def arr(g):
    n = g.contents.Np
    return [np.ctypeslib.as_array(getattr(g.contents, c), shape=(max(n, 1),))[:n].tolist() for c in "xyz"]
out = {"V": sub.contents.V, "pos": arr(sub), "rand": arr(sub.contents.rand)}
print(json.dumps(out))
"""


def write_mock(path):
    x, y, z = uniform_box(11, NPART, L)
    rng = np.random.default_rng(11)  # velocities (km/s): any reproducible values do
    v = rng.standard_normal((3, NPART)) * 300.0
    with open(path, "w") as fh:
        for p in range(NPART):
            fh.write(f"{x[p]:.6f} {y[p]:.6f} {z[p]:.6f} {v[0, p]:.4f} {v[1, p]:.4f} {v[2, p]:.4f} 1.0 0 0\n")


def read_dl(path):
    rows = [ln.split() for ln in open(path) if ln.strip() and not ln.startswith("#")]
    return np.array([[float(t) for t in r[1:]] for r in rows])


def main():
    if not available() or not all(os.path.exists(os.path.join(REF, d)) for d in ("Psb", "Pss", "DLsb", "DLss")):
        sys.exit("reference build missing: run `make -C oracle ref` first")
    out = {"params": np.array([NG, L, NSUB, ALPHA, DK, A])}
    with tempfile.TemporaryDirectory() as tmp:
        indir, outdir = os.path.join(tmp, "in"), os.path.join(tmp, "out")
        os.makedirs(indir)
        os.makedirs(os.path.join(outdir, f"a{A:.4f}_{ID:04d}"))
        mock = os.path.join(indir, f"a{A:.4f}_{ID:04d}.mock")
        write_mock(mock)
        common = [str(NG), str(L), str(NSUB), "FFTW_ESTIMATE"]
        tail = [indir, f"{A}", str(ID), outdir]
        env = dict(os.environ)
        env.pop("GSL_RNG_SEED", None)
        for drv in ("Psb", "Pss"):
            subprocess.run([os.path.join(REF, drv)] + common + [str(ALPHA), str(DK)] + tail, check=True, env=env,
                           stderr=subprocess.DEVNULL)
        for drv in ("DLsb", "DLss"):
            subprocess.run([os.path.join(REF, drv)] + common + tail, check=True, env=env, stderr=subprocess.DEVNULL)
        res = os.path.join(outdir, f"a{A:.4f}_{ID:04d}")
        for drv, tag, kind in (("Psb", "sb", "box"), ("Pss", "ss", "sphere")):
            out[f"{drv}_pl"] = read_table(os.path.join(res, f"Pl_rsd1_los001_{tag}000.txt"))
            out[f"{drv}_pmu"] = read_table(os.path.join(res, f"Pmu_rsd1_los001_{tag}000.txt"))
            r = subprocess.run([sys.executable, "-c", _FIRST_SUB, ROOT, mock, kind, str(L), str(NSUB), str(ALPHA),
                                f"{A}"], check=True, env=env, capture_output=True, text=True)
            sub = json.loads(r.stdout.strip().splitlines()[-1])
            out[f"{drv}_sub_V"] = np.array(sub["V"])
            out[f"{drv}_sub_pos"] = np.array(sub["pos"])
            out[f"{drv}_sub_rand"] = np.array(sub["rand"])
        for drv in ("DLsb", "DLss"):
            for il, los in enumerate(LOS6):
                out[f"{drv}_los{il}"] = read_dl(os.path.join(res, f"{drv}_los{los[0]}{los[1]}{los[2]}.txt"))
        cat = subprocess.run([sys.executable, "-c", r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from oracle.reflib import RefLib
lib = RefLib.lib()
g = lib.gal_loadqpm_cubic(sys.argv[2].encode(), float(sys.argv[3]))
n = g.contents.Np
print(json.dumps([np.ctypeslib.as_array(getattr(g.contents, c), shape=(n,)).tolist() for c in "xyz"]))
""", ROOT, mock, str(L)], check=True, capture_output=True, text=True)
        out["catalog"] = np.array(json.loads(cat.stdout.strip().splitlines()[-1]))
    out["los6"] = np.array(LOS6, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "drivers_small.npz"), **out)
    print("wrote", os.path.join(HERE, "drivers_small.npz"))


if __name__ == "__main__":
    main()
