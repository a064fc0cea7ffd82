"""The 60-operator table, Euler geometry, common-line angles and ASU folding:
oracle and library host code against the golden table of
icosprocess/SRC/icos2f_sym_mat.f90 and analytic properties."""
import numpy as np
import pytest


def test_golden_table_is_the_icosahedral_group(golden_ops):
    R = golden_ops
    assert R.shape == (60, 3, 3)
    for m in R:
        assert np.allclose(m @ m.T, np.eye(3), atol=1e-12)
        assert abs(np.linalg.det(m) - 1) < 1e-12
    # closure: every product is in the set
    flat = R.reshape(60, 9)
    for a in R[::7]:
        for b in R[::5]:
            d = np.abs(flat - (a @ b).reshape(1, 9)).max(axis=1)
            assert d.min() < 1e-12


def test_oracle_ops_match_golden_table_in_order(orc, golden_ops):
    assert np.abs(orc.icos_ops("f64") - golden_ops).max() < 1e-13
    # FP32: the table's 14-digit decimals and the exact values round to the same floats
    assert np.array_equal(orc.icos_ops("f32"), golden_ops.astype(np.float32))


def test_library_ops_match_golden_table_in_order(built, golden_ops):
    import cryoim_gb300 as ci
    assert np.array_equal(ci.icos_ops(), golden_ops.astype(np.float32))


def test_generator_order_is_a_permutation_of_the_table(orc, golden_ops):
    g = orc.icos_gen("f64")
    used = set()
    for m in golden_ops:
        d = np.abs(g.reshape(60, 9) - m.reshape(1, 9)).max(axis=1)
        k = int(np.argmin(d))
        assert d[k] < 1e-12
        used.add(k)
    assert len(used) == 60


@pytest.mark.parametrize("fp", ["f32", "f64"])
def test_euler_matrix_zyz(orc, fp):
    from synth import euler_mat
    for th, ph, om in [(0, 0, 0), (30, 40, 50), (90, -45, 270), (123.4, 200.1, -33.3)]:
        m = orc.euler(th, ph, om, fp)
        tol = 1e-6 if fp == "f32" else 1e-13
        assert np.abs(m - euler_mat(th, ph, om)).max() < tol


def test_crosslin_angles_define_common_lines(orc):
    """alpha1/alpha2 are the in-plane angles of the shared line v = z1 x S z2: rotating
    (cos a1, sin a1, 0) by R1 and (cos a2, sin a2, 0) by S R2 both give v."""
    from synth import euler_mat
    o1, o2 = (75.0, 12.0, 40.0), (81.0, -20.0, 200.0)
    a1, a2 = orc.crosslin(o1, o2, "f64")
    ops = orc.icos_ops("f64")
    R1, R2 = euler_mat(*o1), euler_mat(*o2)
    nvalid = 0
    for j in range(60):
        z1, z2a = R1[:, 2], ops[j] @ R2[:, 2]
        v = np.cross(z1, z2a)
        if np.linalg.norm(v) < 0.5:
            assert a1[j] == 1000 and a2[j] == 1000
            continue
        nvalid += 1
        v /= np.linalg.norm(v)
        l1 = R1 @ [np.cos(np.radians(a1[j])), np.sin(np.radians(a1[j])), 0]
        l2 = ops[j] @ R2 @ [np.cos(np.radians(a2[j])), np.sin(np.radians(a2[j])), 0]
        assert np.allclose(l1, v, atol=1e-9) and np.allclose(l2, v, atol=1e-9)
    assert nvalid > 30


def test_asu_fold_is_idempotent_and_equivalent(orc):
    from synth import euler_mat, in_asu
    rng = np.random.default_rng(1)
    ops = orc.icos_ops("f64")
    for _ in range(50):
        o = (rng.uniform(0, 180), rng.uniform(-180, 180), rng.uniform(-180, 180))
        f = orc.asu_fold(*o, fp="f64")
        f2 = orc.asu_fold(*f, fp="f64")
        assert np.allclose(f, f2, atol=1e-9)
        Rf = euler_mat(*f)
        assert in_asu(Rf[:, 2]) or abs(Rf[2, 2]) < 1e-9
        # f is S*R(o) for some operator S
        Ro = euler_mat(*o)
        assert min(np.abs(S @ Ro - Rf).max() for S in ops) < 1e-8


def test_library_asu_fold_matches_oracle_fp32(orc, built):
    import cryoim_gb300 as ci
    rng = np.random.default_rng(2)
    for _ in range(30):
        o = (float(rng.uniform(0, 180)), float(rng.uniform(-180, 180)), float(rng.uniform(0, 360)))
        a = ci.asu_fold(*o)
        b = orc.asu_fold(*o, fp="f32")
        assert np.allclose(a, b, atol=2e-3), (o, a, b)


def test_equalort_and_frame_transforms(orc, built):
    """proc_icos equalort / transform_ort_2fTo5f / 2fTo3f: library (FP32) against the
    oracle (FP32) and against the defining rotation in FP64."""
    import cryoim_gb300 as ci
    from synth import euler_mat
    e_lib = ci.equalort(70.0, 10.0, 33.0)
    e_orc = orc.equalort(70.0, 10.0, 33.0, "f32")
    assert np.abs(e_lib - e_orc).max() < 1e-3
    # every equivalent orientation is S*R for a group element S
    R = euler_mat(70.0, 10.0, 33.0)
    ops = orc.icos_ops("f64")
    for t, p, o in e_lib.astype(np.float64):
        Re = euler_mat(t, p, o)
        assert min(np.abs(S @ R - Re).max() for S in ops) < 1e-4
    th = np.array([10.0, 70.0, 120.0]); ph = np.array([5.0, -30.0, 100.0]); om = np.array([0.0, 45.0, 300.0])
    for to in (5, 3):
        a = ci.transform_ort(to, th, ph, om)
        b = orc.transform_ort(to, th, ph, om, "f32")
        for x, y in zip(a, b):
            assert np.abs(x - y).max() < 1e-3
        d2r = np.pi / 180
        if to == 5:
            v = np.arccos(np.cos(60 * d2r) / np.sin(36 * d2r))
            rot0 = np.array([[np.cos(v), 0, np.sin(v)], [0, 1, 0], [-np.sin(v), 0, np.cos(v)]])
        else:
            w = np.arccos(np.cos(36 * d2r) / np.sin(60 * d2r))
            rot0 = np.array([[1, 0, 0], [0, np.cos(-w), np.sin(-w)], [0, -np.sin(-w), np.cos(-w)]])
        for i in range(3):
            want = rot0 @ euler_mat(th[i], ph[i], om[i])
            got = euler_mat(float(a[0][i]), float(a[1][i]), float(a[2][i]))
            assert np.abs(want - got).max() < 1e-4
