"""Copies the reference's own output snapshots into tests/golden/reference_runs/.

galax-cli --out writes the final body state of a run as a GALX v1 snapshot
(galax-cli/src/main.rs:343-352, galax-io/src/lib.rs:21-42).  The reference
repository ships three such files (runs/demo/snap_0010.bin, runs/test/snap_0005.bin,
runs/viz-demo/snap_0010.bin, N = 1000 each); they are the only force values the
reference itself produced that exist here, so they are kept as fixtures (the
reference tree is not available where the tests run).

    python tests/golden/copy_reference_runs.py [reference_root]
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
RUNS = {"demo_snap_0010.bin": "runs/demo/snap_0010.bin",
        "test_snap_0005.bin": "runs/test/snap_0005.bin",
        "viz-demo_snap_0010.bin": "runs/viz-demo/snap_0010.bin"}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    out = os.path.join(HERE, "reference_runs")
    os.makedirs(out, exist_ok=True)
    for dst, src in RUNS.items():
        shutil.copyfile(os.path.join(root, src), os.path.join(out, dst))
        print(dst)


if __name__ == "__main__":
    main()
