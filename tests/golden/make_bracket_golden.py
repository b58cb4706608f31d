"""Golden fixtures of the BRK-A-01 set-up, made by the reference's own code.

    python tests/golden/make_bracket_golden.py <path of the reference checkout>

Imports the reference's create_bracket_domain (src/am/core/geometry.py:79-196)
and create_brk_a_01_static_case_1/2 (src/am/core/loads.py:163-306) and records,
at several resolutions, the voxel grid, the load ring's nodes, the force vectors
(nonzero entries) and the constrained DOFs into bracket_golden.npz beside this
file.  Tests read only the .npz."""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RESOLUTIONS = (12.0, 5.0, 4.0, 3.0, 2.5, 2.0)


def main(ref: str) -> None:
    sys.path.insert(0, ref)
    from src.am.core.geometry import create_bracket_domain
    from src.am.core.loads import create_brk_a_01_static_case_1, create_brk_a_01_static_case_2

    out = {"resolutions": np.array(RESOLUTIONS)}
    for r in RESOLUTIONS:
        dom = create_bracket_domain(resolution_mm=r)
        nx, ny, nz = dom.shape
        N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
        key = f"r{r:g}"
        out[f"{key}_grid"] = dom.grid
        for c, fn in ((1, create_brk_a_01_static_case_1), (2, create_brk_a_01_static_case_2)):
            lc = fn(dom.shape, r)
            F = lc.get_force_vector(N)
            nzi = np.flatnonzero(F)
            out[f"{key}_c{c}_F_idx"] = nzi.astype(np.int64)
            out[f"{key}_c{c}_F_val"] = F[nzi]
            out[f"{key}_c{c}_total"] = np.asarray(lc.distributed_loads[0].total_force, dtype=np.float64)
            if c == 1:
                out[f"{key}_ring"] = np.asarray(lc.distributed_loads[0].node_indices, dtype=np.int64)
                out[f"{key}_fixed"] = lc.get_constrained_dofs().astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "bracket_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "bracket_golden.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
