"""Regenerates the golden fixtures in this folder from the AutoPDEx source tree.

Run in a container that has the reference checkout (it is not needed to run the tests):
    python tests/golden/make_golden.py /path/to/AutoPDEx

* cook_q2_mesh.npz: the inline Q2 Cook-membrane mesh of
  tests/test_user_elem_impl_diff_and_adaptive_load_step.py:31-55 (x_nodes, elements,
  surface_elements), parsed from the file as data.
* golden.json: the golden scalars asserted by the reference's tests on this path (the Q2 Cook
  solution's u.u, its first derivatives with respect to Young's modulus E and Poisson's ratio
  nu, and its second derivatives d2/dE2, d2/dE dnu, d2/dnu dE, d2/dnu2).
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    src = open(os.path.join(ref, "tests", "test_user_elem_impl_diff_and_adaptive_load_step.py")).read()

    def grab(name):
        m = re.search(name + r" = jnp\.array\((\[.*?\])\)\n", src, re.S)
        # the literal is a nested list of numbers; parse it with numpy after stripping brackets
        txt = m.group(1)
        rows = re.findall(r"\[([^\[\]]*)\]", txt)
        return np.array([[float(v) for v in r.split(",") if v.strip()] for r in rows])

    x = grab("x_nodes")
    e = grab("elements").astype(np.int64)
    s = grab("surface_elements").astype(np.int64)
    np.savez(os.path.join(HERE, "cook_q2_mesh.npz"), x_nodes=x, elements=e, surface_elements=s)
    g1 = re.search(r"isclose\(test, ([0-9.]+)\)", open(os.path.join(ref, "tests", "test_dicts_as_dofs_user_potential.py")).read())
    # test1 .. test7 of the reference test: u.u, its first and its second derivatives in E and nu
    g2 = re.findall(r"jnp\.array\((-?[0-9.]+), dtype=jnp\.float64\)", src)
    golden = {
        "poisson_5x5_sum_phi": {"value": float(g1.group(1)),
                                "source": "tests/test_dicts_as_dofs_user_potential.py:63"},
        "cook_q2_dofs_dot_dofs": {"value": float(g2[0]),
                                  "source": "tests/test_user_elem_impl_diff_and_adaptive_load_step.py:153"},
        "cook_q2_d_dofs_dot_dofs_d_youngs_modulus": {
            "value": float(g2[1]), "source": "tests/test_user_elem_impl_diff_and_adaptive_load_step.py:154"},
        "cook_q2_d_dofs_dot_dofs_d_poisson_ratio": {
            "value": float(g2[2]), "source": "tests/test_user_elem_impl_diff_and_adaptive_load_step.py:155"},
    }
    # test4 .. test7: second derivatives (E E, E nu, nu E, nu nu), lines 156-159
    for k, name in enumerate(("youngs_modulus_youngs_modulus", "youngs_modulus_poisson_ratio",
                              "poisson_ratio_youngs_modulus", "poisson_ratio_poisson_ratio")):
        golden["cook_q2_d2_dofs_dot_dofs_d_" + name] = {
            "value": float(g2[3 + k]),
            "source": "tests/test_user_elem_impl_diff_and_adaptive_load_step.py:%d" % (156 + k)}
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(golden, fh, indent=1)
    print(golden)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the AutoPDEx source tree>")
    main(sys.argv[1])
