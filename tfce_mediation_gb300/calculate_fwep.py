"""Drop-ins for the 1-p(FWER) image scripts:
tfce_mediation/tmanalysis/calculate_fweP_vertex.py:37-79 and
tfce_mediation/tmanalysis/calculate_fweP_voxel.py:23-62.

Both read a TFCE image and the permutation maxima CSV, and write the 1-p(FWE)
image next to the reference's names: for every value x > 0,
1-p = max(idx - 1, 0) / N with idx = #{null < x} (the sorted null's
left insertion point), 0 elsewhere.  The sort and the per-vertex lookups run
on the device (fwer_sort, fwer_lookup); image I/O is io.load_* / io.save_*.

    python -m tfce_mediation_gb300.calculate_fwep vertex -i img_TFCE.mgh perm.csv [-l]
    python -m tfce_mediation_gb300.calculate_fwep voxel  -i img_TFCE.nii.gz perm.csv [-l]
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from .fwer import accuracy, fwep
from .io import load_mgh, load_nifti, save_mgh, save_nifti


def parser(ap=None, ext="*.mgh"):
    ap = ap or argparse.ArgumentParser(description="Calculate 1-P[FWE] from max TFCE values from randomisation.")
    ap.add_argument("-i", "--input", nargs=2, metavar=(ext, "*.csv"), help="[tfce_image] [perm_tfce_max]",
                    required=True)
    ap.add_argument("-l", "--outputneglog10", help="Outputs the -log10(FWEp) image", action="store_true")
    return ap


def vertex_run(opts):
    """calculate_fweP_vertex.run: writes <image>_FWEcorrP.mgh (and, with -l,
    <image>_FWEneglog10p.mgh) beside the input image; returns the 1-p values
    of the vertices with TFCE > 0."""
    img_path, csv_path = str(opts.input[0]), str(opts.input[1])
    null = np.genfromtxt(csv_path, delimiter=",")
    data_full, affine = load_mgh(img_path, with_affine=True)
    stem = img_path.split(".mgh", 1)[0]
    data = np.squeeze(data_full)
    bin_mask = data > 0
    corrp = fwep(data[bin_mask], null)
    outmask = np.zeros_like(data_full)
    outmask[bin_mask, 0, 0] = corrp
    save_mgh(outmask, affine, "%s_FWEcorrP.mgh" % stem)
    print("The accuracy is p = 0.05 +/- %.4f" % accuracy(null.shape[0]))
    if opts.outputneglog10:
        with np.errstate(divide="ignore"):
            outmask[bin_mask, 0, 0] = -np.log10(1 - corrp)
        save_mgh(outmask, affine, "%s_FWEneglog10p.mgh" % stem)
    return corrp


def voxel_run(opts):
    """calculate_fweP_voxel.run: writes <name>_FWEcorrP.nii.gz in the working
    directory (and, with -l, <name>_FWEneglog10p.mgh, the reference's name
    for that image); returns the 1-p image."""
    img_path, csv_path = str(opts.input[0]), str(opts.input[1])
    null = np.genfromtxt(csv_path, delimiter=",")
    data, affine = load_nifti(img_path)
    corrp = np.zeros(data.shape)
    thresh = data > 0
    corrp[thresh] = fwep(data[thresh], null)
    name = os.path.splitext(os.path.splitext(os.path.basename(img_path))[0])[0]
    print("The accuracy is p = 0.05 +/- %.4f" % accuracy(null.shape[0]))
    save_nifti(corrp, affine, "%s_FWEcorrP.nii.gz" % name)
    if opts.outputneglog10:
        with np.errstate(divide="ignore"):
            save_mgh((-np.log10(1 - corrp)).astype(np.float32), affine, "%s_FWEneglog10p.mgh" % name)
    return corrp


def main(argv=None):
    top = argparse.ArgumentParser(description="1-P[FWE] images from permutation maxima (GPU lookups)")
    sub = top.add_subparsers(dest="space", required=True)
    parser(sub.add_parser("vertex"), "*.mgh")
    parser(sub.add_parser("voxel"), "*.nii.gz")
    opts = top.parse_args(argv)
    return vertex_run(opts) if opts.space == "vertex" else voxel_run(opts)


if __name__ == "__main__":
    main()
