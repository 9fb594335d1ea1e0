"""User potentials through the C++ drop-in API on the GPU, against the reference.

tests/cpp/test_gpu_api.cpp writes the potentials the way a user of the reference does
(GlobalPotential::add_potential with MappedWorkspace lambdas, add_dof, NewtonsMethod).
  * contact: the step problem (tet4_6p) plus a cubic ground-contact potential that is active
    only below the plane (a conditional potential, the idiom of
    examples/dynamic_elasticity_with_contact.cpp:126-139) and a second DoF set of handles tied
    to the mesh by springs (one potential couples both DoF sets).  Against the reference's
    energy, gradient and NewtonsMethod::solve of the same problem (tests/golden/tet4_6p_contact.npz):
    energy 1e-12, gradient 1e-9 of max |g|; FP64: same Newton iterations, CG within 3 %,
    positions and handles within 1e-8 of their displacement; mixed: within 1e-6.
  * mixed derivatives: NewtonsMethod::parameter_gradient (the adjoint's symbolically generated
    -lambda . dg/dp kernels) for mu and lambda against the reference's own gradient() of the
    element gradient (tests/golden/mixed_nh_tet4.npz), 1e-12 relative.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


@pytest.mark.parametrize("precision", [0, 1])
def test_conditional_contact_and_second_dof_set_match_reference(gpu_api_test, golden, tmp_path, precision):
    from problem_io import contact_scene, write_problem, write_scene

    from symx_gb300 import problems

    p = problems.step_problem("tet4_6p")
    scene = contact_scene(p)
    write_problem(tmp_path / "p.bin", p)
    write_scene(tmp_path / "s.bin", scene)
    r = subprocess.run([gpu_api_test, "contact", str(tmp_path / "p.bin"), str(tmp_path / "s.bin"), str(tmp_path),
                        str(precision)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    ref = golden("tet4_6p_contact")
    E = np.fromfile(tmp_path / "E.bin")[0]
    g = np.fromfile(tmp_path / "grad.bin")
    assert abs(E - ref["E"]) <= 1e-12 * abs(ref["E"])
    assert g.size == ref["grad"].size == 3 * (p["X"].shape[0] + 3)
    assert np.max(np.abs(g - ref["grad"])) <= 1e-9 * np.max(np.abs(ref["grad"]))
    ret, newton, cg, res = open(tmp_path / "stats.txt").read().split()
    assert int(ret) == 0 and float(res) < 1e-6
    x = np.fromfile(tmp_path / "x_final.bin").reshape(-1, 3)
    h = np.fromfile(tmp_path / "h_final.bin").reshape(-1, 3)
    tol = 1e-8 if precision == 0 else 1e-6
    assert np.linalg.norm(x - ref["x_full"]) / np.linalg.norm(ref["x_full"] - p["x0"]) < tol
    assert np.linalg.norm(h - ref["h_full"]) / np.linalg.norm(ref["h_full"] - scene["handle"]) < tol
    if precision == 0:
        assert int(newton) == int(ref["newton_iterations"])
        assert abs(int(cg) - int(ref["cg_iterations"])) <= 2 + 0.03 * int(ref["cg_iterations"])
    # the contact is active at the solution: vertices below the plane
    assert np.sum(x[:, 1] < scene["ground_y"]) > 0


def test_mixed_derivative_kernels_match_reference_symbolic(gpu_api_test, golden, tmp_path):
    from problem_io import write_problem

    from symx_gb300 import problems

    p = problems.step_problem("tet4_6p")
    write_problem(tmp_path / "p.bin", p)
    lam_adj = problems.normal(61, 3 * p["X"].shape[0])
    lam_adj.tofile(tmp_path / "l.bin")
    r = subprocess.run([gpu_api_test, "mixed", str(tmp_path / "p.bin"), str(tmp_path / "l.bin"), str(tmp_path / "o.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(tmp_path / "o.bin")
    ne = p["conn"].shape[0]
    d_mu, d_lam = out[:ne], out[ne:]
    ref = golden("mixed_nh_tet4")
    le = lam_adj.reshape(-1, 3)[p["conn"]].reshape(ne, 12)
    ref_mu = -np.sum(le * ref["dg_dmu_tet4_6p"], axis=1)
    ref_lam = -np.sum(le * ref["dg_dlam_tet4_6p"], axis=1)
    assert np.max(np.abs(d_mu - ref_mu)) <= 1e-12 * np.max(np.abs(ref_mu))
    assert np.max(np.abs(d_lam - ref_lam)) <= 1e-12 * np.max(np.abs(ref_lam))
