"""tests/unit/math.test.mjs of the reference, restated for the Python
mirror's Vec3 and Mat4: products, inverses, rigid rotations and the
right-hand rule, lookAt, and the range checks (ValueError
where the reference throws RangeError)."""

import math

import pytest

from raymond_gb300 import Mat4, Vec3


def random(seed):
    """The fixed sequence math.test.mjs:7-12 draws from: a 32-bit LCG mapped to
    [-10, 10). Python's integers are exact, as the reference's doubles are
    below 2**53 here."""
    def nxt():
        nonlocal seed
        seed = (seed * 1664525 + 1013904223) % 4294967296
        return seed / 4294967296 * 20.0 - 10.0
    return nxt


def random_matrix(nxt):
    return Mat4(*[nxt() for _ in range(16)])


def rows(r):
    return Mat4(*[x for row in r for x in row])


def assert_matrix_close(a, b, eps=1e-9):
    for r in range(4):
        for c in range(4):
            assert abs(a.value(r, c) - b.value(r, c)) <= eps, (r, c)


def test_multiply_mat4_matches_the_textbook_product():
    nxt = random(1)
    for _ in range(50):
        a, b = random_matrix(nxt), random_matrix(nxt)
        product = a.multiplyMat4(b)
        for r in range(4):
            for c in range(4):
                expected = sum(a.value(r, k) * b.value(k, c) for k in range(4))
                assert abs(product.value(r, c) - expected) <= 1e-9


def test_inverse_undoes_a_matrix():
    nxt = random(2)
    for _ in range(50):
        m = random_matrix(nxt)
        assert_matrix_close(m.multiplyMat4(m.inverse()), Mat4.identity(), 1e-6)


def test_translate_moves_points_but_not_directions():
    t = Mat4.translate(1, 2, 3)
    assert t.multiplyVector3(Vec3(10, 20, 30)).tuple() == (11, 22, 33)
    assert t.multiplyDirection(Vec3(10, 20, 30)).tuple() == (10, 20, 30)


@pytest.mark.parametrize("rot", [Mat4.rotateX, Mat4.rotateY, Mat4.rotateZ])
def test_rotations_are_rigid_and_compose_by_adding_angles(rot):
    for theta in (0.0, 0.5, 1.0, 2.5, -1.2):
        r = rot(theta)
        assert abs(r.determinant() - 1.0) <= 1e-9
        inv = r.inverse()
        for i in range(4):
            for j in range(4):
                assert abs(inv.value(i, j) - r.value(j, i)) <= 1e-9
    assert_matrix_close(rot(0.3).multiplyMat4(rot(0.4)), rot(0.7))


@pytest.mark.parametrize("rot,src,dst", [(Mat4.rotateZ, (1, 0, 0), (0, 1, 0)),
                                         (Mat4.rotateX, (0, 1, 0), (0, 0, 1)),
                                         (Mat4.rotateY, (0, 0, 1), (1, 0, 0))])
def test_rotations_follow_the_right_hand_rule(rot, src, dst):
    v = rot(math.pi / 2.0).multiplyDirection(Vec3(*src))
    for got, want in zip((v.x, v.y, v.z), dst):
        assert abs(got - want) <= 1e-9


def test_inverse_raises_for_a_singular_matrix():
    with pytest.raises(ValueError):
        Mat4.scale(1, 0, 1).inverse()


def test_elements_outside_the_matrix_are_refused():
    m = Mat4.identity()
    for call in (lambda: m.value(4, 0), lambda: m.value(0, -1), lambda: m.setValue(0, 4, 1)):
        with pytest.raises(ValueError):
            call()
    m.setValue(2, 3, 7.5)
    assert m.value(2, 3) == 7.5


def test_look_at_points_minus_z_at_the_target():
    eye, target = Vec3(3, 4, 12), Vec3(0, 1, 0)
    m = Mat4.lookAt(eye, target, Vec3(0, 1, 0))
    origin = m.multiplyVector3(Vec3(0, 0, 0))
    assert (origin.x, origin.y, origin.z) == eye.tuple()
    forward = m.multiplyDirection(Vec3(0, 0, -1))
    expected = target.subtract(eye).normalized()
    for got, want in zip((forward.x, forward.y, forward.z), expected.tuple()):
        assert abs(got - want) <= 1e-9
    assert m.multiplyDirection(Vec3(0, 1, 0)).y > 0.0
    assert abs(m.multiplyDirection(Vec3(1, 0, 0)).y) <= 1e-9  # right is level
    assert abs(m.determinant() - 1.0) <= 1e-9


def test_vec3_arithmetic():
    a, b = Vec3(1, 2, 3), Vec3(4, 5, 6)
    assert a.add(b).tuple() == (5, 7, 9)
    assert b.subtract(a).tuple() == (3, 3, 3)
    assert Vec3(1, 0, 0).cross(Vec3(0, 1, 0)).tuple() == (0, 0, 1)
    assert a.dot(b) == 32
    assert abs(Vec3(3, 4, 12).length() - 13.0) <= 1e-9
    assert abs(b.normalized().length() - 1.0) <= 1e-9
    c = Vec3(1, -2, 3)
    assert c.scale(2).tuple() == (2, -4, 6)
    assert c.multiply(Vec3(2, 3, 4)).tuple() == (2, -6, 12)
    assert c.negate().tuple() == (-1, 2, -3)
    assert c.lerp(Vec3(3, 2, -1), 0.5).tuple() == (2, 0, 1)


def test_transpose_swaps_rows_and_columns():
    m = rows([[1, 2, 3, 4], [5, 6, 7, 8], [9, 10, 11, 12], [13, 14, 15, 16]])
    t = m.transpose()
    for r in range(4):
        for c in range(4):
            assert t.value(r, c) == m.value(c, r)
