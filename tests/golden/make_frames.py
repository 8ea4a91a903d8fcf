"""Make tests/golden/reference_frames.npz from the reference's own configuration files.

The reference ships equilibrated and lattice water frames as .xyz files (input_coords/,
input_files/). The GPU parity tests run on those frames, but the reference tree is not present
where they run, so this script reads them once, with the engine library's reader
(pimd_read_config_header + pimd_read_xyz, read_method 1 as the reference's default) checked
number for number against the oracle's restatement of the same format, and stores the box and
the centred coordinates as float64 arrays together with the SHA-256 of each source file.

    python tests/golden/make_frames.py [reference_dir]   (default: $PIMD_REFERENCE_DIR)
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# name -> path inside the reference tree
FRAMES = {
    "input_32": "input_coords/input_32.xyz",     # 32 H2O, L = 9.85467 A
    "input_128": "input_coords/input_128.xyz",   # 128 H2O, L = 15.658825 A
    "input_512": "input_coords/input_512.xyz",   # 512 H2O, L = 24.832313 A
    "4nm": "input_files/4nm.xyz",                # 2228 H2O, L = 40.5855 A
}
OUT = os.path.join(HERE, "reference_frames.npz")


def main(ref):
    import __graft_entry__ as ge
    import state_io_oracle as so

    pkg = ge.load_package()
    pkg.build_lib.build()
    out = {}
    for name, rel in FRAMES.items():
        path = os.path.join(ref, rel)
        box, RRc = pkg.state_io.read_xyz(path, read_method=1)
        obox, oRRc = so.read_xyz(path, read_method=1)
        assert np.array_equal(box, obox) and np.array_equal(RRc, oRRc), name
        out[name + "_box"] = box
        out[name + "_RRc"] = RRc
        out[name + "_sha256"] = np.array(hashlib.sha256(open(path, "rb").read()).hexdigest())
        print("%-10s %5d atoms  box %s" % (name, len(RRc), box))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PIMD_REFERENCE_DIR")
    if not ref:
        sys.exit("give the reference directory as an argument or in PIMD_REFERENCE_DIR")
    main(ref)
