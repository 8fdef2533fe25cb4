"""Regenerates the committed fixtures under tests/golden/.

* ``sigma_kat.npz`` -- the reference's own sigma^2(R) tables (cosmo_files/sig0.npz and
  cosmo_files/Del2k.npz, produced by cosmo_files/sigmas.py:239-248 with cosmolopy): the full
  Delta^2(k) table and every 10th radius of sig0.  Needs a checkout of the reference: its
  path comes from ``--reference DIR`` or the ``ES_REFERENCE_DIR`` environment variable (only
  this script reads it); without one, this fixture is left as committed.
* ``oracle_32.npz`` -- FP64 oracle outputs for seeded 32^3 boxes (centre and sphere modes,
  delta_T and P(k)), so the oracle itself is pinned against regressions and the GPU tests have
  a fixed target.

Run from the repository root:  python tests/golden/make_golden.py [--reference DIR]
"""
import argparse
import importlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))


def sigma_kat(ref_dir):
    cosmo_files = os.path.join(ref_dir, "cosmo_files")
    a = np.load(os.path.join(cosmo_files, "sig0.npz"))
    b = np.load(os.path.join(cosmo_files, "Del2k.npz"))
    np.savez_compressed(os.path.join(HERE, "sigma_kat.npz"), k=b["k"], Del2=b["Del2"],
                        radius=a["radius"][::10], sig0=a["sig0"][::10], mass=a["mass"][::10])


def oracle_32():
    cos = importlib.import_module("21cmpy_gb300.cosmology")
    sch = importlib.import_module("21cmpy_gb300.schedule")
    grf = importlib.import_module("21cmpy_gb300.grf")
    from oracle import es_oracle as O
    n, L, z = 32, 48.0, 8.0
    d = grf.density_box(n, L, seed=0, z=z)
    out = {"density": d}
    for name, kw in [("center", {}), ("sphere", {"update": 1, "R_max": 10.0})]:
        args = dict(zeta=30.0, t_vir_min=1e4, R_max=15.0, cosmo=cos.BASELINE_COSMO)
        args.update(kw)
        st = sch.ionize_setup(n, L, z, **args)
        r = O.conv_bubbles(d, st)
        out[f"{name}_ionized"] = r["ionized"]
        out[f"{name}_exempt"] = np.packbits(r["exempt"])
        out[f"{name}_radii"] = st.radii()
        out[f"{name}_denoms"] = st.denoms()
    c = cos.brightness_temperature_factor(z, cos.BASELINE_COSMO)
    xh = (1.0 - out["center_ionized"]).astype(np.float32)
    dT, ave = O.delta_T(xh, d, c)
    edges = sch.pk_edges(n, L, 20)
    K, k_ave, ps_ave, cnt = O.power_spectrum(dT, ave, L, edges)
    out.update(dT=dT, ave=np.float64(ave), K=K, k_ave=k_ave, ps_ave=ps_ave, count=cnt)
    np.savez_compressed(os.path.join(HERE, "oracle_32.npz"), **out)


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description="regenerate tests/golden fixtures")
    ap.add_argument("--reference", default=os.environ.get("ES_REFERENCE_DIR"),
                    help="checkout of the reference repository (for sigma_kat.npz)")
    args = ap.parse_args()
    if args.reference and os.path.isdir(os.path.join(args.reference, "cosmo_files")):
        sigma_kat(args.reference)
    else:
        print("no reference checkout given (--reference / ES_REFERENCE_DIR): sigma_kat.npz left as committed")
    oracle_32()
    print("fixtures written to", HERE)
