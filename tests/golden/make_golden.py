"""Regenerate the golden fixtures in this folder from the MATLAB reference's own data.

The reference (project-asgard/DG-SparseGrid) cannot run here (no MATLAB or Octave), so its
committed gold files are the executable-free pins for the oracle.  This script reads them
once, in the container that has the reference checked out, and packs the subset the
``apply_A`` hot path needs into small ``.npz`` files that travel with the tests:

* ``two_scale_rel.npz``   -- H0/G0/scale_co/phi_co of ``two_scale/two_scale_rel_{1..8}.mat``
                             (the multiwavelet filters ``OperatorTwoScale_wavelet2.m:18-26`` loads)
* ``element_table.npz``   -- ``gold/generated-inputs/element_table/{table,ids}_{1,2,3}d_{SG,FG}.dat``
                             and ``1d_index_*.dat`` (``gold/gold_hash_table.m:11-80``)
* ``connectivity.npz``    -- ``connect_1_{2,3,8}.dat``, ``connect_n_2_3_FG_*.dat``,
                             ``connect_n_3_4_SG_*.dat`` (``gold/gold_connect.m:19-57``)
* ``permutations.npz``    -- ``gold/generated-inputs/permutations/*`` (``gold/gold_permute.m``)
* ``quadrature.npz``      -- ``gold/generated-inputs/quadrature/*`` (``gold/gold_quadrature.m``)
* ``transformations.npz`` -- ``operator_two_scale_*.dat``, ``multiwavelet_*.dat``, ``combine_dim_*.dat``
* ``coefficients.npz``    -- ``gold/generated-inputs/coefficients/{continuity2,3,6,diffusion2}_coefficients_l*``
                             (one level set each; ``gold/gold_coefficients.m``)
* ``basis.npz``           -- ``gold/generated-inputs/basis/transform_blocks_*`` (``gold/gold_basis.m``)
* ``pde.npz``             -- ``gold/generated-inputs/pde/{continuity2,continuity_3,continuity_6,diffusion_2}_*``
                             (``gold/gold_pde.m``)
* ``adapt.npz``           -- ``gold/generated-inputs/adapt/continuity{1,2,3}_*`` (``gold/gold_adapt.m``)
* ``time_advance.npz``    -- RK3 and backward-Euler trajectories ``continuity{1,2,3,6}_*``, ``diffusion2_*``
                             and the adaptive ``continuity2_ad_*``, ``diffusion2_ad_implicit_*`` ``_t{0..4}.dat``
                             (``gold/gold_time_advance.m:252-364``)

Run:  python tests/golden/make_golden.py <reference_root>
      (or set ASG_REFERENCE_ROOT; the path of the DG-SparseGrid checkout is required)
"""
import glob
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_octave_text(path):
    """Parse the ``write_octave_like_output.m`` format: '#' header lines, then rows."""
    rows = None
    cols = None
    data = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#"):
                m = re.match(r"#\s*rows:\s*(\d+)", line)
                if m:
                    rows = int(m.group(1))
                m = re.match(r"#\s*columns:\s*(\d+)", line)
                if m:
                    cols = int(m.group(1))
                continue
            s = line.strip()
            if s:
                data.extend(float(v) for v in s.split())
    arr = np.array(data, dtype=np.float64)
    if rows is not None and cols is not None:
        if rows * cols == 0:
            return np.zeros((rows, cols))
        arr = arr.reshape(rows, cols)
    return arr


def main(ref_root):
    gold = os.path.join(ref_root, "gold", "generated-inputs")

    # ---- two-scale filters -------------------------------------------------------------
    import scipy.io as sio

    ts = {}
    for deg in range(1, 9):
        m = sio.loadmat(os.path.join(ref_root, "two_scale", "two_scale_rel_%d.mat" % deg))
        for key in ("H0", "G0", "scale_co", "phi_co"):
            ts["%s_%d" % (key, deg)] = np.asarray(m[key], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "two_scale_rel.npz"), **ts)

    def pack(subdir, pattern, outname, keyfn=None):
        out = {}
        for path in sorted(glob.glob(os.path.join(gold, subdir, pattern))):
            name = os.path.basename(path)[:-4]
            key = keyfn(name) if keyfn else name
            out[key] = read_octave_text(path)
        np.savez_compressed(os.path.join(HERE, outname), **out)
        return len(out)

    n = 0
    n += pack("element_table", "*.dat", "element_table.npz")
    out = {}
    for pat in ("connect_1_*.dat", "connect_n_2_3_FG_*.dat", "connect_n_3_4_SG_*.dat"):
        for path in sorted(glob.glob(os.path.join(gold, "connectivity", pat))):
            out[os.path.basename(path)[:-4]] = read_octave_text(path)
    np.savez_compressed(os.path.join(HERE, "connectivity.npz"), **out)
    n += len(out)
    n += pack("permutations", "*.dat", "permutations.npz")
    n += pack("quadrature", "*.dat", "quadrature.npz")
    out = {}
    for pat in ("operator_two_scale_*.dat", "multiwavelet_*.dat", "combine_dim_*.dat"):
        for path in sorted(glob.glob(os.path.join(gold, "transformations", pat))):
            out[os.path.basename(path)[:-4]] = read_octave_text(path)
    np.savez_compressed(os.path.join(HERE, "transformations.npz"), **out)
    n += len(out)
    out = {}
    # wavelet-space 1-D operators pde.terms{t}.terms_1D{d}.mat (gold/gold_coefficients.m,
    # central flux), one level set per configuration PDE
    for stem in ("continuity2_coefficients_l4_4_d3", "continuity3_coefficients_l2_3_2_d4",
                 "continuity6_coefficients_l2_2_2_2_2_2_d4", "diffusion2_coefficients_l2_3_d5"):
        for path in sorted(glob.glob(os.path.join(gold, "coefficients", stem + "_*_*.dat"))):
            out[os.path.basename(path)[:-4]] = read_octave_text(path)
    np.savez_compressed(os.path.join(HERE, "coefficients.npz"), **out)
    n += len(out)
    out = {}
    # the transform's blocks (gold/gold_basis.m: OperatorTwoScale_wavelet2 at levels 2, 5
    # and degrees 2, 5)
    for path in sorted(glob.glob(os.path.join(gold, "basis", "transform_blocks_*.dat"))):
        out[os.path.basename(path)[:-4]] = read_octave_text(path)
    np.savez_compressed(os.path.join(HERE, "basis.npz"), **out)
    n += len(out)
    out = {}
    # PDE specifications evaluated at x = 0.1..0.5, t = 5 (gold/gold_pde.m): initial
    # conditions, exact solutions, sources and dt of the configurations' PDEs
    for pat in ("continuity2_*.dat", "continuity_3_*.dat", "continuity_6_*.dat", "diffusion_2_*.dat"):
        for path in sorted(glob.glob(os.path.join(gold, "pde", pat))):
            out[os.path.basename(path)[:-4]] = read_octave_text(path)
    np.savez_compressed(os.path.join(HERE, "pde.npz"), **out)
    n += len(out)
    out = {}
    # adaptation of given vectors (gold/gold_adapt.m:1-14, 60-112): original, coarsened and
    # refined vectors, and the tables as [levels, cells] rows
    for path in sorted(glob.glob(os.path.join(gold, "adapt", "continuity*_l*_d*_*.dat"))):
        out[os.path.basename(path)[:-4]] = read_octave_text(path)
    np.savez_compressed(os.path.join(HERE, "adapt.npz"), **out)
    n += len(out)
    out = {}
    for stem in ("continuity1_sg_l2_d2", "continuity1_sg_l4_d3", "continuity1_fg_l2_d2",
                 "continuity2_sg_l2_d2", "continuity2_sg_l4_d3", "continuity2_fg_l2_d2",
                 "continuity2_fg_l3_4_d3", "continuity3_sg_l2_d2", "continuity3_sg_l4_d3", "continuity3_sg_l3_4_2_d4",
                 "continuity6_sg_l2_d2", "continuity6_sg_l2_d3", "continuity6_sg_l2_3_2_3_3_2_d2",
                 # backward Euler (gold/gold_time_advance.m:156-173, 237-240)
                 "continuity1_implicit_l2_d2", "continuity1_implicit_l4_d3", "continuity2_implicit_l2_d2",
                 "continuity2_implicit_l4_d3", "continuity2_implicit_fg_l3_4_d3",
                 # LDG diffusion with inhomogeneous Dirichlet data (gold_time_advance.m:40-51, 179-193, 203-234)
                 "diffusion2_sg_l2_d2", "diffusion2_sg_l3_d3", "diffusion2_sg_l4_d4", "diffusion2_sg_l4_5_d2",
                 "diffusion2_implicit_sg_l3_d3", "diffusion2_implicit_sg_l4_d3", "diffusion2_implicit_sg_l5_d3",
                 "diffusion2_implicit_sg_l4_5_d2",
                 # adaptive runs (gold/gold_time_advance.m:21-34, 291-362)
                 "continuity2_ad_sg_l3_d4", "diffusion2_ad_implicit_sg_l3_d4"):
        for t in range(5):
            path = os.path.join(gold, "time_advance", "%s_t%d.dat" % (stem, t))
            out["%s_t%d" % (stem, t)] = read_octave_text(path).reshape(-1)
    np.savez_compressed(os.path.join(HERE, "time_advance.npz"), **out)
    n += len(out)
    print("packed %d gold arrays into %s" % (n, HERE))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ASG_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <reference_root>  (or set ASG_REFERENCE_ROOT)")
    main(root)
