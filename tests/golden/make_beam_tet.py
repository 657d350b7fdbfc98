"""Regenerate tests/golden/beam_tet.npz from the reference's data/beam-tet.mesh.

The reference's A-form MMS test (test/integration/test_aform_source.cpp:80)
reads data/beam-tet.mesh: 48 tets on [0,8]x[0,1]^2 with boundary attributes
1..3.  This script reads that MFEM ASCII file once, in the container that has
the reference mounted, and stores its arrays so that tests run without it.
Usage: python tests/golden/make_beam_tet.py /path/to/reference/data/beam-tet.mesh
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", ".."))
from hephaestus_gb300.meshes import read_mfem_tet_mesh  # noqa: E402

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_beam_tet.py <reference checkout>/data/beam-tet.mesh")
src = sys.argv[1]
verts, tets, btris, battr, eattr = read_mfem_tet_mesh(src)
out = os.path.join(os.path.dirname(__file__), "beam_tet.npz")
np.savez(out, verts=verts, tets=tets, btris=btris, battr=battr, eattr=eattr)
print(out, verts.shape, tets.shape, btris.shape, np.bincount(battr))
