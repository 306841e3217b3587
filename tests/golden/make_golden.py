"""Regenerate the oracle regression fixtures in this directory.

The reference publishes no golden vectors for the Poisson path and cannot be
built here, so these fixtures pin the oracle's restatement against its own
earlier outputs (grid, FormMetrics iaj, the assembled operator and the
mean-removed right-hand side) on two small seeded grids.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "oracle"), os.path.join(REPO, "vfs-wind_gb300")]

import oracle as O  # noqa: E402
from vfs_poisson import configs as CF  # noqa: E402


def make(name, case):
    d = O.dims_of(case)
    met = O.form_metrics(d, case.coor)
    lhs = O.poisson_lhs(d, case.nvert, met)
    b = O.rhs(d, case.nvert, lhs["gid"], case.ucont, met["aj"])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), coor=case.coor, vol=lhs["vol"], b=b, iaj=met["iaj"])


if __name__ == "__main__":
    make("channel_8", CF.channel(8, 8, 8))
    make("cylinder_12", CF.cylinder(12, 8, 12))
    print("written")
