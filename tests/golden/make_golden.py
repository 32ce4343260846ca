"""Generate the golden fixtures of this directory from the reference tree.

Run once in a container that has the reference checkout (path given as the
first argument); the GPU machine does not.  It copies the reference's own test
inputs and outputs for the Chebyshev path into small files:

  ts_profile.npy      TStest/profile.0 (= test/profile.0, same md5): the FSC
                      Tollmien-Schlichting mean profile, rows y rho u v w T
  cases.json          run parameters of each case (from its input.dat /
                      *.inp) and the reference's published eigenvalues
                      (test/space.1:3, TStest/README.md:9-10,
                      thesis/TStest/time.ref:2, space.ref:3)
  space1.ref          test/space.1 (spatial N=32 eigenfunction)
  thesis_time.ref     thesis/TStest/time.ref (temporal N=96 eigenfunction)
  thesis_space.ref    thesis/TStest/space.ref (spatial N=96 eigenfunction)
  *.inp               the stdin files of those runs, verbatim: test/input.dat,
                      TStest/input.dat, thesis/TStest/temporal.inp, spatial.inp
  cf_*, fsc_*         CFtest and FSCtest (curved wall, curve = 2): input.dat,
                      profile.0 (as .npy), space.ref, and their eigenvalues
                      (CFtest/README.md, the header of FSCtest/space.ref)
"""
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_input(path):
    vals = []
    for ln in open(path):
        f = ln.split("!")[0].replace(",", " ").split()
        if f:
            vals.append(f)
    mattyp = int(vals[0][0])
    o = 1
    T0 = 0.0
    if mattyp == 1:
        T0 = float(vals[1][0]); o = 2
    Ma, Re, Pr = map(float, vals[o][:3])
    ny, yi, ymax = int(vals[o + 1][0]), float(vals[o + 1][1]), float(vals[o + 1][2])
    ievec = int(vals[o + 2][0])
    ider = int(vals[o + 3][0])
    top, wall, wallt, curve = map(int, vals[o + 4][:4])
    itype = int(vals[o + 5][0])
    a = complex(float(vals[o + 6][0]), float(vals[o + 6][1]))
    b = complex(float(vals[o + 7][0]), float(vals[o + 7][1]))
    d = dict(mattyp=mattyp, T0=T0, Ma=Ma, Re=Re, Pr=Pr, ny=ny, yi=yi, ymax=ymax, ievec=ievec, ider=ider,
             top=top, wall=wall, wallt=wallt, curve=curve, itype=itype)
    if itype == 1:
        d["alpha"], d["beta"], d["omega"] = [a.real, a.imag], [b.real, b.imag], [0.0, 0.0]
    else:
        d["omega"], d["beta"], d["alpha"] = [a.real, a.imag], [b.real, b.imag], [0.0, 0.0]
    return d


def main(ref):
    rows = []
    for ln in open(os.path.join(ref, "TStest", "profile.0")):
        if ln[:1] == "#" or not ln.split():
            continue
        rows.append([float(t) for t in ln.split()[:6]])
    np.save(os.path.join(HERE, "ts_profile.npy"), np.asarray(rows, dtype=np.float64))
    cases = {}
    c = read_input(os.path.join(ref, "test", "input.dat"))
    c["golden"] = [2.2805022654496E-01, -6.5136925762007E-03]
    c["eigfunction"] = "space1.ref"
    cases["test_spatial_n32"] = c
    c = read_input(os.path.join(ref, "TStest", "input.dat"))
    c64 = dict(c, ny=64, golden=[2.2804739410500E-01, -6.5163146761218E-03])
    cases["tstest_spatial_n64"] = c64
    cases["tstest_spatial_n96"] = dict(c, golden=[2.2804739411367E-01, -6.5163146912049E-03])
    c = read_input(os.path.join(ref, "thesis", "TStest", "temporal.inp"))
    c["golden"] = [1.1467880189410E-01, 2.3844535276599E-03]
    c["eigfunction"] = "thesis_time.ref"
    cases["thesis_temporal_n96"] = c
    c = read_input(os.path.join(ref, "thesis", "TStest", "spatial.inp"))
    c["golden"] = [2.2804739411180E-01, -6.5163146952626E-03]
    c["eigfunction"] = "thesis_space.ref"
    cases["thesis_spatial_n96"] = c
    # curved-wall crossflow and Falkner-Skan-Cooke cases (curve = 2, circh):
    # their own profiles; eigenvalues from CFtest/README.md (SGI at N = 64,
    # MacOS at N = 96) and the header of FSCtest/space.ref
    for tag, sub, gold in (("cf", "CFtest", {64: [-3.7392297537875E+001, -2.9982641664422E-001],
                                              96: [-3.7392546274473E+001, -2.9977113927779E-001]}),
                           ("fsc", "FSCtest", {64: [-4.6108596548503E-001, -7.0050272583092E-003]})):
        rows = []
        for ln in open(os.path.join(ref, sub, "profile.0")):
            if ln[:1] == "#" or not ln.split():
                continue
            rows.append([float(t.replace("D", "E").replace("d", "e")) for t in ln.split()[:6]])
        np.save(os.path.join(HERE, f"{tag}_profile.npy"), np.asarray(rows, dtype=np.float64))
        shutil.copyfile(os.path.join(ref, sub, "input.dat"), os.path.join(HERE, f"{tag}_input.inp"))
        shutil.copyfile(os.path.join(ref, sub, "space.ref"), os.path.join(HERE, f"{tag}_space.ref"))
        c = read_input(os.path.join(ref, sub, "input.dat"))
        c["x"] = 500.0          # the station read after the index (the circle's radius for curve = 2)
        for ny, g in gold.items():
            e = dict(c, ny=ny, golden=g, profile=f"{tag}_profile.npy")
            if ny == 64:
                e["eigfunction_rows"] = f"{tag}_space.ref"
            cases[f"{tag}test_spatial_n{ny}"] = e
    with open(os.path.join(HERE, "cases.json"), "w") as fh:
        json.dump(cases, fh, indent=1)
    for src, dst in [("test/input.dat", "test_input.inp"), ("TStest/input.dat", "tstest_input.inp"),
                     ("thesis/TStest/temporal.inp", "thesis_temporal.inp"),
                     ("thesis/TStest/spatial.inp", "thesis_spatial.inp")]:
        shutil.copyfile(os.path.join(ref, src), os.path.join(HERE, dst))
    shutil.copyfile(os.path.join(ref, "test", "space.1"), os.path.join(HERE, "space1.ref"))
    shutil.copyfile(os.path.join(ref, "thesis", "TStest", "time.ref"), os.path.join(HERE, "thesis_time.ref"))
    shutil.copyfile(os.path.join(ref, "thesis", "TStest", "space.ref"), os.path.join(HERE, "thesis_space.ref"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference tree>")
    main(sys.argv[1])
