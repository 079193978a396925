"""Generates the golden fixtures in this folder from the CPU restatement
(oracle/), so that the GPU tests can compare against them on a machine where
the oracle is not re-run, and so that the oracle itself is pinned against
drift.  Run from the repository root:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from gturbo3d_gb300.synth import forcing_amplitude, initial_potential  # noqa: E402
from oracle.gturbo_oracle import (Oracle, Params, fluxes, glob, helicity, iniforcing,  # noqa: E402
                                  defk, rann_stream, spectrum)

SEED0 = 8299396   # the reference's files/seed.000 value


def trace(name, n, forcing, dt2_mode, steps=(1, 2, 5), **phys):
    p = Params(nx=n[0], ny=n[1], nz=n[2], forcing=forcing, dt2_mode=dt2_mode, **phys)
    o = Oracle(p)
    if forcing != "none":
        p.famp = forcing_amplitude(0.1, o.fm.nf)
        o = Oracle(p)
    b0 = initial_potential(*n, 0)
    out = {"b0": np.stack(b0), "seed0": SEED0, "famp": p.famp, "shape": np.array(n)}
    n1 = o.nlt(b0, b0)
    out["nlt_b0"] = np.stack(n1)
    g = glob(b0, p, o.wk)
    out["glob_energy"] = g["energy"]
    out["glob_enstrophy"] = g["enstrophy"]
    out["helicity"] = helicity(b0, p, o.wk)
    sp, sp2 = spectrum(b0, p, o.wk)
    out["spectrum"], out["spectrum2d"] = sp, sp2
    out["flux"] = fluxes(b0, n1, p, o.wk)
    b, s, done = b0, SEED0, 0
    for k in steps:
        b, s = o.run(b, s, k - done)
        done = k
        out[f"b_{k}"] = np.stack(b)
        out[f"seed_{k}"] = s
    np.savez_compressed(HERE / f"{name}.npz", **out)


def main():
    vals, s = rann_stream(SEED0, 1000)
    np.savez_compressed(HERE / "lcg_seed0.npz", values=vals, final=s, seed=SEED0)
    fm = {}
    for kind in ("3d3c", "2d2c"):
        p = Params(nx=64, ny=64, nz=64, forcing=kind, famp=1.0)
        m = iniforcing(p, defk(p))
        fm[f"{kind}_ix"], fm[f"{kind}_iy"], fm[f"{kind}_iz"], fm[f"{kind}_ff"] = m.ix, m.iy, m.iz, m.ff
    np.savez_compressed(HERE / "forced_modes_64.npz", **fm)
    trace("trace16_3d3c_rk2", (16, 16, 16), "3d3c", "rk2")
    trace("trace16_2d2c_as_built", (16, 16, 16), "2d2c", "as_built")
    trace("trace_32x16x8_3d3c_rk2", (32, 16, 8), "3d3c", "rk2", nu=5e-3, omega=2.0)


if __name__ == "__main__":
    main()
