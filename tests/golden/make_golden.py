"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own CpuPropagator<double> (compiled from its headers into
oracle/_ref/libcp3ref.so by oracle/Makefile) on a fixed list of cases and
stores inputs plus outputs as .npz.  It needs the reference sources, so it runs
only on the machine that has them; the fixtures it writes are committed and the
tests read those.

    REF_DIR=<reference source directory> python tests/golden/make_golden.py
"""
import argparse
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cudaprob3_gb300 import grids as G  # noqa: E402


def strided(n, k):
    """About k indices spread over range(n), always with both ends."""
    idx = np.unique(np.round(np.linspace(0, n - 1, min(k, n))).astype(np.int64))
    return idx


def case(name, cos, en, radii, rhos, ye, params, height=22.0, anti=False, kc=None, ke=None,
         note=""):
    rho_eff = (np.asarray(rhos) * np.asarray(ye)) / 0.5
    p = oracle.ref_calculate(cos, en, radii, rho_eff, params, height, anti)
    ic = strided(len(cos), kc) if kc else np.arange(len(cos))
    ie = strided(len(en), ke) if ke else np.arange(len(en))
    sub = p[:, ic][:, :, ie]
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, cosines=np.asarray(cos, np.float64), energies=np.asarray(en, np.float64),
                        radii=np.asarray(radii, np.float64), rhos=np.asarray(rhos, np.float64),
                        ye=np.asarray(ye, np.float64), params=np.asarray(params, np.float64),
                        height_km=np.float64(height), anti=np.int32(anti), idx_c=ic, idx_e=ie,
                        probs=sub, note=np.str_(note))
    print("%-28s %4d x %4d -> %d pairs stored" % (name, len(cos), len(en), sub.shape[1] * sub.shape[2]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=os.environ.get("REF_DIR"),
                    help="the reference's source directory (default: $REF_DIR)")
    a = ap.parse_args()
    if not a.ref_dir:
        sys.exit("set REF_DIR (or --ref-dir) to the reference's source directory")
    oracle.build(a.ref_dir)
    if not oracle.ref_available():
        sys.exit("reference library not built; fixtures need the reference sources")
    P4, P12 = G.PREM_4, G.PREM_12
    nom = G.NOMINAL
    c256, e256 = G.linspace(-1.0, 0.0, 256), G.logspace(0.5, 100.0, 256)
    for anti in (False, True):
        tag = "nubar" if anti else "nu"
        case("prem4_256_" + tag, c256, e256, P4.radii, P4.rhos, P4.ye, nom, anti=anti,
             kc=40, ke=40, note="4-shell body, 256x256 grid, 0.5-100 GeV")
        c, e = G.linspace(-1.0, 0.0, 128), G.logspace(0.1, 1000.0, 128)
        case("prem12_128_" + tag, c, e, P12.radii, P12.rhos, P12.ye, nom, anti=anti,
             kc=48, ke=48, note="11-shell body, 128x128 grid, 0.1-1000 GeV")
    # Electron fraction 0.5 everywhere: identical to the reference's fixed factor.
    case("prem4_256_ye05", c256, e256, P4.radii, P4.rhos, np.full(5, 0.5), nom, kc=40, ke=40,
         note="ye=0.5: probe values P(mu->mu)[0][0], [255][255], P(mu->e)[128][128]")
    ragged_c = np.concatenate([G.linspace(-1.0, 1.0, 37)])
    ragged_e = G.logspace(0.1, 1000.0, 53)
    case("prem12_ragged_37x53", ragged_c, ragged_e, P12.radii, P12.rhos, P12.ye, nom,
         note="cosines over [-1, 1] (upgoing half crosses only the atmosphere)")
    case("prem12_dm12_zero", G.linspace(-1, 0, 24), G.logspace(0.1, 100, 31), P12.radii,
         P12.rhos, P12.ye, (nom[0], nom[1], nom[2], nom[3], 0.0, nom[5]),
         note="dm21=0: degeneracy break of propagator.hpp:233-236")
    case("prem12_dm23_zero", G.linspace(-1, 0, 24), G.logspace(0.1, 100, 31), P12.radii,
         P12.rhos, P12.ye, (nom[0], nom[1], nom[2], nom[3], nom[4], 0.0), note="dm32=0")
    case("prem12_inverted", G.linspace(-1, 0, 24), G.logspace(0.1, 100, 31), P12.radii,
         P12.rhos, P12.ye, (nom[0], nom[1], nom[2], nom[3], nom[4], -2.6e-3),
         note="inverted ordering")
    case("prem12_inverted_nubar", G.linspace(-1, 0, 24), G.logspace(0.1, 100, 31), P12.radii,
         P12.rhos, P12.ye, (nom[0], nom[1], nom[2], nom[3], nom[4], -2.6e-3), anti=True,
         note="inverted ordering, antineutrino")
    desc = slice(None, None, -1)
    case("prem4_descending", G.linspace(-1, 0, 20), G.logspace(0.5, 100, 20), P4.radii[desc],
         P4.rhos[desc], P4.ye[desc], nom, note="radii given outside-in (no flip)")
    case("no_center_row", G.linspace(-1, 0, 20), G.logspace(0.5, 100, 20),
         [1220.0, 3480.0, 5701.0, 6371.0], [13.0, 11.3, 5.0, 3.3], [0.468, 0.468, 0.497, 0.497],
         nom, note="no radius-0 row: the innermost shell is crossed at c=-1")
    case("one_shell", G.linspace(-1, 0.2, 17), G.logspace(0.5, 100, 19), [6371.0], [4.5], [0.5],
         nom, note="single shell")
    case("height_0km", G.linspace(-1, 1, 21), G.logspace(0.5, 100, 19), P4.radii, P4.rhos, P4.ye,
         nom, height=0.0, note="production height 0")
    case("height_100km", G.linspace(-1, 1, 21), G.logspace(0.5, 100, 19), P4.radii, P4.rhos,
         P4.ye, nom, height=100.0, note="production height 100 km")
    sets = G.draw_parameter_sets(6, seed=0)
    for k, ps in enumerate(sets):
        case("prem12_set%d" % k, G.linspace(-1, 0, 40), G.logspace(0.1, 1000, 40), P12.radii,
             P12.rhos, P12.ye, tuple(ps), anti=bool(k % 2), note="parameter set %d of seed 0" % k)
    mpath = os.path.join(a.ref_dir, "example", "models", "PREM_59layer.dat")
    if os.path.exists(mpath):
        r59, d59 = G.read_density_file(mpath)
        case("prem59", G.linspace(-1, 0, 64), G.logspace(0.1, 1000, 48), r59, d59,
             np.where(r59 <= 3480.0, 0.468, 0.497), nom, note="59-row PREM table")
    density_files(a.ref_dir)


# the density models shipped with the reference (example/models), copied as
# fixtures, and two variants of the 12-layer file for the edge cases of the
# two-column read loop (propagator.hpp:169-184)
MODELS = ("PREM_4layer.dat", "PREM_10layer.dat", "PREM_12layer.dat", "PREM_59layer.dat")
MODELS_DIR = os.path.join(HERE, "models")


def density_files(ref_dir):
    """Goldens of the reference's setDensityFromFile on each model file, on the
    grid of tests/cpp/dropin_example.cpp (37 cosines in [-1, 0] x 45 energies
    over 0.5-100 GeV, nominal parameters, neutrinos): the rows the reference
    reads are stored as radii/rhos (ye 0.5, its fixed factor), so the files
    also serve the setDensity path."""
    os.makedirs(MODELS_DIR, exist_ok=True)
    for m in MODELS:
        shutil.copyfile(os.path.join(ref_dir, "example", "models", m), os.path.join(MODELS_DIR, m))
    with open(os.path.join(MODELS_DIR, "PREM_12layer.dat")) as f:
        rows = f.read().splitlines()
    # trailing blank lines and spaces: skipped by the stream extraction
    with open(os.path.join(MODELS_DIR, "PREM_12layer_trailing_blank.dat"), "w") as f:
        f.write("\n".join(rows) + "\n\n   \n\n")
    # the rows outside-in (setDensity accepts either order) with a text row
    # after the eighth: the read loop stops there, so the body is the eight
    # outermost rows (no radius-0 row: the innermost is crossed as a full chord)
    desc = [r for r in rows if r.strip()][::-1]
    with open(os.path.join(MODELS_DIR, "PREM_12layer_stops_at_text.dat"), "w") as f:
        f.write("\n".join(desc[:8] + ["end of the mantle rows"] + desc[8:]) + "\n")
    c, e = G.linspace(-1.0, 0.0, 37), G.logspace(0.5, 100.0, 45)
    for name in sorted(os.listdir(MODELS_DIR)):
        path = os.path.join(MODELS_DIR, name)
        radii, rhos = G.read_density_file(path)
        probs = oracle.ref_calculate_file(c, e, path, G.NOMINAL, 22.0, False)
        out = os.path.join(HERE, "file_" + name[:-4] + ".npz")
        np.savez_compressed(out, cosines=c, energies=e, radii=radii, rhos=rhos, ye=np.full(radii.size, 0.5),
                            params=np.asarray(G.NOMINAL, np.float64), height_km=np.float64(22.0),
                            anti=np.int32(0), idx_c=np.arange(c.size), idx_e=np.arange(e.size), probs=probs,
                            density_file=np.str_(name),
                            note=np.str_("the reference's setDensityFromFile on models/" + name))
        print("%-40s %2d rows -> %d pairs stored" % (os.path.basename(out), radii.size, c.size * e.size))


if __name__ == "__main__":
    main()
