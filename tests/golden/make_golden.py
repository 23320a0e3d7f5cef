"""Copy the reference's own test fixtures that pin the forward path into
tests/golden/.

Run in a container where the reference checkout is present:

    python tests/golden/make_golden.py /path/to/reference

Forward cases (<case>/): the CRMod inputs (elem.dat, elec.dat, rho.dat,
crmod.cfg) and the CRMod output volt.dat of a reference tomodir.  The
measurement configurations are the (strnr, vnr) columns of volt.dat.
Inversion cases add the tomodir's crtomo.cfg, CRTomo's inv.ctr and the
model and data files written after iteration 1 (rho01.mag, rho01.pha,
volt01.dat; minimal also rho02.mag and the coverage and uncertainty files
of src/bbsens.f90 and src/bmcm_mod.f90).

CutMcK cases (cutmck_<case>/): the grid before (elem.dat.orig, elec.dat.orig)
and after (elem.dat, elec.dat) the reference's Cuthill-McKee renumbering.

The files are data fixtures of the reference's tests/ and examples/ trees,
copied byte for byte.
"""
import os
import shutil
import sys

FORWARD = {
    # name: (tomodir, pin note)
    "minimal": "tests/minimal/Reference",
    "testmodinv": "tests/TestModInv/Reference",
    "mixed_surf": "tests/2.5D_mixed_surf/Reference",
    "decoupling_2d_sink": "tests/GridDecoupling/regular_grids/01_no_decoupling",
}

# inversion cases: the CRTomo configuration and its control output inv.ctr
# (src/kont2.f90), added to the forward case of the same tomodir, whose
# volt.dat is the inverted data set
INVERSION = {
    "minimal": "tests/minimal/Reference",
    "mixed_surf": "tests/2.5D_mixed_surf/Reference",
}

# DC_Problem: one mesh and data set inverted twice by the reference, as a
# complex problem (crtomo.cfg, inv.ctr) and with the DC routines (ldc:
# crtomo_dc.cfg, inv_dc.ctr, a run that the DC factor ended with errnr 28)
DC_PROBLEM = "tests/DC_Problem"

# a robust DC inversion (examples/DifferenceInversion/02/time0): its
# crtomo.cfg, grid, data and the inv.ctr of its run
ROBUST_DC = "examples/DifferenceInversion/02/time0"

# a robust DC difference inversion (examples/DifferenceInversion/02/time1)
# against the reference state of time0: its data (d0.dat), final model
# (m0.mag = time0's rho05.mag) and that model's response (fm0.dat =
# time0's volt05.dat); the grid is time0's
DIFF_DC = "examples/DifferenceInversion/02"

# data noise (src/make_noise.f90, src/rdati.f90:110-140, 257-290): the clean
# data, the noise model (crt.noisemod, seed 1) and the noise the reference drew
NOISE = "examples/MGS/01_simple/03_mgs"

CUTMCK = {
    "minimal": "tests/minimal/Reference/grid",
    "mixed_surf": "tests/2.5D_mixed_surf/Reference/grid",
    "decoupling": "tests/GridDecoupling/regular_grids/GRID",
    "rect_complex": "examples/Grids/Rectangular/02_complex/grid",
    "mgs_advanced": "examples/MGS/02_advanced/GRID",
    "error_parameters": "tests/error_parameters/skeleton_files/grid",
}


def main(ref: str):
    here = os.path.dirname(os.path.abspath(__file__))
    for name, d in FORWARD.items():
        out = os.path.join(here, name)
        os.makedirs(out, exist_ok=True)
        src = os.path.join(ref, d)
        for f in ("grid/elem.dat", "grid/elec.dat", "rho/rho.dat", "exe/crmod.cfg", "mod/volt.dat"):
            shutil.copyfile(os.path.join(src, f), os.path.join(out, os.path.basename(f)))
        with open(os.path.join(out, "SOURCE"), "w") as fh:
            fh.write(d + "\n")
    for name, d in INVERSION.items():
        out = os.path.join(here, name)
        src = os.path.join(ref, d)
        for f in ("exe/crtomo.cfg", "inv/inv.ctr", "inv/rho01.mag", "inv/rho01.pha", "inv/volt01.dat"):
            shutil.copyfile(os.path.join(src, f), os.path.join(out, os.path.basename(f)))
        if name == "minimal":
            # rho02.mag, the coverage and the uncertainty files (mswitch 15)
            for f in ("rho02.mag", "coverage.mag", "coverage.mag_fpi", "ata.diag", "ata.diag_fpi",
                      "ata_reg.diag", "cov1_m.diag", "res_m.diag", "cov2_m.diag"):
                shutil.copyfile(os.path.join(src, "inv", f), os.path.join(out, f))
    out = os.path.join(here, "dc_problem")
    os.makedirs(out, exist_ok=True)
    src = os.path.join(ref, DC_PROBLEM)
    for f, dst in (("Complex/grid/elem.dat", "elem.dat"), ("Complex/grid/elec.dat", "elec.dat"),
                   ("Complex/mod/volt.dat", "volt.dat"), ("Complex/exe/crtomo.cfg", "crtomo.cfg"),
                   ("Complex/inv/inv.ctr", "inv.ctr"), ("DC/exe/crtomo.cfg", "crtomo_dc.cfg"),
                   ("DC/inv/inv.ctr", "inv_dc.ctr")):
        shutil.copyfile(os.path.join(src, f), os.path.join(out, dst))
    with open(os.path.join(out, "SOURCE"), "w") as fh:
        fh.write(DC_PROBLEM + "/{Complex,DC}\n")
    out = os.path.join(here, "robust_dc")
    os.makedirs(out, exist_ok=True)
    src = os.path.join(ref, ROBUST_DC)
    for f in ("grid/elem.dat", "grid/elec.dat", "mod/volt.dat", "exe/crtomo.cfg", "inv/inv.ctr"):
        shutil.copyfile(os.path.join(src, f), os.path.join(out, os.path.basename(f)))
    with open(os.path.join(out, "SOURCE"), "w") as fh:
        fh.write(ROBUST_DC + "\n")
    out = os.path.join(here, "diff_dc")
    os.makedirs(out, exist_ok=True)
    src = os.path.join(ref, DIFF_DC)
    for f, dst in (("time1/exe/crtomo.cfg", "crtomo.cfg"), ("time1/mod/volt1.dat", "volt.dat"),
                   ("time1/inv/inv.ctr", "inv.ctr"), ("time0/mod/volt.dat", "d0.dat"),
                   ("time0/inv/rho05.mag", "m0.mag"), ("time0/inv/volt05.dat", "fm0.dat")):
        shutil.copyfile(os.path.join(src, f), os.path.join(out, dst))
    with open(os.path.join(out, "SOURCE"), "w") as fh:
        fh.write(DIFF_DC + "/{time0,time1}; grid: tests/golden/robust_dc (the same elem.dat, elec.dat)\n")
    out = os.path.join(here, "noise_mgs")
    os.makedirs(out, exist_ok=True)
    src = os.path.join(ref, NOISE)
    for f in ("mod/volt.dat", "exe/crt.noisemod", "exe/inv.mynoise_rho", "exe/inv.mynoise_pha",
              "exe/inv.mynoise_voltages"):
        shutil.copyfile(os.path.join(src, f), os.path.join(out, os.path.basename(f)))
    with open(os.path.join(out, "SOURCE"), "w") as fh:
        fh.write(NOISE + "/{mod,exe}\n")
    for name, d in CUTMCK.items():
        out = os.path.join(here, "cutmck_" + name)
        os.makedirs(out, exist_ok=True)
        src = os.path.join(ref, d)
        for f in ("elem.dat.orig", "elec.dat.orig", "elem.dat", "elec.dat"):
            shutil.copyfile(os.path.join(src, f), os.path.join(out, f))
        with open(os.path.join(out, "SOURCE"), "w") as fh:
            fh.write(d + "\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
