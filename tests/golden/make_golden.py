"""Generate the golden fixtures in this folder from SEM2DPACK's examples.

Run in a container where the reference checkout is available:

    python tests/golden/make_golden.py /path/to/sem2dpack

It reads the reference's own test data (nothing is written from memory):
  EXAMPLES/LambsProblem/{Ux,Uz}_file_ascii   analytic traces (EX2DDIR),
                                              pass threshold 0.005
                                              (LambsProblem/analyze_test.m:21-22)
  EXAMPLES/LambsProblem/test.out             recorded misfits of the reference
  EXAMPLES/TestSH/uyref.mat                   analytic SH trace (SEMLAB),
                                              threshold 0.02 (TestSH/analyze_test.m:14-15)
  EXAMPLES/Anisotropic/p{1..4}.tab            reference output at stations
                                              4, 18, 23, 46 (Anisotropic/write_seis.m)
  EXAMPLES/InaBox/info                        check-mode log: npoin, dt, nt
  EXAMPLES/{LambsProblem,TestSH,Anisotropic,InaBox,
           TestFlt2D_SCEC_TPV3_inplane,RateState,TestFlt1D,
           Bimaterial_fault,2.5D_V-shape_rate-and-state,2.5D_inplane,
           2D_roughness_drag_approximation,Kelvin_Visco_FZ,
           Velocity_weakening}/Par.inp
                                              the input decks, as text (parinp_*)
  EXAMPLES/RateState/{Ux,Vx,Tau}_{0,3,6,9}km_ascii
                                              the reference's slip, slip rate and shear
                                              stress change every step at x = 0, 3, 6,
                                              9 km of its rate-and-state deck
                                              (RateState/Par.inp; provenance of the
                                              traces not recorded: a loose check)
  EXAMPLES/**/Par*.inp (the others)           the decks the front end refuses, as text
                                              (refused_*)
  EXAMPLES/TestAbso/data_mat/{stacey,paraxial}_PSV.mat
                                              the reference's misfits of the direct
                                              P (errp) and S (errs) waves against
                                              incidence angle (theta) on a bottom
                                              boundary with Stacey P3 or
                                              Clayton-Engquist P1 conditions
                                              (TestAbso/test_abso_PSV.m:95-136)
and writes golden.npz.  The GPU machine and the test suite only read the npz.
"""
import os
import re
import sys

import numpy as np


def main(ref):
    ex = os.path.join(ref, "EXAMPLES")
    out = {}
    lamb = os.path.join(ex, "LambsProblem")
    out["lamb_ux"] = np.loadtxt(os.path.join(lamb, "Ux_file_ascii"))
    out["lamb_uz"] = np.loadtxt(os.path.join(lamb, "Uz_file_ascii"))
    txt = open(os.path.join(lamb, "test.out")).read()
    m = re.search(r"misfit ux1 ux2 uz1 uz2 = ([0-9.eE+\- ]+)", txt)
    out["lamb_recorded_misfit"] = np.array([float(v) for v in m.group(1).split()])

    from scipy.io import loadmat
    sh = loadmat(os.path.join(ex, "TestSH", "uyref.mat"))
    out["sh_tref"] = np.asarray(sh["tref"], dtype=np.float64).ravel()
    out["sh_uref"] = np.asarray(sh["uref"], dtype=np.float64).ravel()

    for k in range(1, 5):
        out["aniso_p%d" % k] = np.loadtxt(os.path.join(ex, "Anisotropic", "p%d.tab" % k))
    out["aniso_stations"] = np.array([4, 18, 23, 46])

    info = open(os.path.join(ex, "InaBox", "info")).read()
    out["inabox_npoin"] = np.array(int(re.search(r"Total number of GLL points[ .]*= *(\d+)", info).group(1)))
    out["inabox_nelem"] = np.array(int(re.search(r"Total number of elements[ .]*= *(\d+)", info).group(1)))
    out["inabox_dt"] = np.array(float(re.search(r"Time step \(secs\) *= *([0-9.E+\-]+)", info).group(1)))
    out["inabox_nt"] = np.array(int(re.search(r"Number of time steps *= *(\d+)", info).group(1)))

    for kind in ("stacey", "paraxial"):
        m = loadmat(os.path.join(ex, "TestAbso", "data_mat", kind + "_PSV.mat"))
        for key in ("theta", "errp", "errs"):
            out["abso_%s_%s" % (kind, key)] = np.asarray(m[key], dtype=np.float64).ravel()

    for q in ("Ux", "Vx", "Tau"):
        out["ratestate_" + q] = np.stack([np.loadtxt(os.path.join(ex, "RateState", "%s_%dkm_ascii" % (q, x)))
                                          for x in (0, 3, 6, 9)])

    for name in ("LambsProblem", "TestSH", "Anisotropic", "InaBox", "TestFlt2D_SCEC_TPV3_inplane", "RateState",
                 "TestFlt1D", "Bimaterial_fault", "2.5D_V-shape_rate-and-state", "2.5D_inplane",
                 "2D_roughness_drag_approximation", "Kelvin_Visco_FZ", "Velocity_weakening", "TestAbso",
                 "TestLayers", "TestLayers_2"):
        text = open(os.path.join(ex, name, "Par.inp")).read()
        out["parinp_" + name] = np.array(text)
        # the tables the deck names (file='...'), as text
        for fname in sorted(set(re.findall(r"""file\s*=\s*['"]([^'"]+)['"]""", text))):
            path = os.path.join(ex, name, fname)
            if os.path.exists(path):
                out["exfile_%s__%s" % (name, fname)] = np.array(open(path).read())

    # the other example decks, which the front end refuses (off the GPU path)
    import glob
    for f in sorted(glob.glob(os.path.join(ex, "**", "Par*.inp"), recursive=True)):
        rel = os.path.relpath(f, ex)
        key = "parinp_" + os.path.dirname(rel).replace("/", "__").replace("+", "_")
        if os.path.basename(rel) != "Par.inp":
            key += "__" + os.path.splitext(os.path.basename(rel))[0]
        if key not in out:
            out["refused_" + key[len("parinp_"):]] = np.array(open(f).read())

    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")
    np.savez_compressed(dst, **out)
    for k, v in out.items():
        print(k, np.shape(v))
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/sem2dpack")
    main(sys.argv[1])
