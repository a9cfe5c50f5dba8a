"""tests/unit/math.test.mjs of the reference, restated for the Python
mirror's Vec3, Vec4 and Mat4: products, inverses, rigid rotations and the
right-hand rule, the projections, lookAt, and the range checks (ValueError
where the reference throws RangeError)."""

import math

import pytest

from raymond_gb300 import Mat4, Vec3, Vec4


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


def test_multiply_vector4_multiplies_a_column_vector():
    m = rows([[1, 2, 3, 4], [5, 6, 7, 8], [9, 10, 11, 12], [13, 14, 15, 16]])
    assert m.multiplyVector4(Vec4(1, 0, -1, 2)).tuple() == (6, 14, 22, 30)
    assert m.row(1).tuple() == (5, 6, 7, 8)
    assert m.column(2).tuple() == (3, 7, 11, 15)


def test_inverse_undoes_a_matrix():
    nxt = random(2)
    for _ in range(50):
        m = random_matrix(nxt)
        assert_matrix_close(m.multiplyMat4(m.inverse()), Mat4.identity(), 1e-6)


def test_translate_moves_points_but_not_directions():
    t = Mat4.translate(1, 2, 3)
    assert t.multiplyVector4(Vec4(10, 20, 30, 1)).tuple() == (11, 22, 33, 1)
    assert t.multiplyVector4(Vec4(10, 20, 30, 0)).tuple() == (10, 20, 30, 0)


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
    v = rot(math.pi / 2.0).multiplyVector4(Vec4(*src, 0))
    for got, want in zip((v.x, v.y, v.z), dst):
        assert abs(got - want) <= 1e-9


def test_inverse_raises_for_a_singular_matrix():
    with pytest.raises(ValueError):
        Mat4.scale(1, 0, 1).inverse()


def test_elements_outside_the_matrix_are_refused():
    m = Mat4.identity()
    for call in (lambda: m.value(4, 0), lambda: m.value(0, -1), lambda: m.setValue(0, 4, 1),
                 lambda: m.row(4), lambda: m.column(-1)):
        with pytest.raises(ValueError):
            call()
    m.setValue(2, 3, 7.5)
    assert m.value(2, 3) == 7.5


def test_orthographic_maps_its_box_to_clip_space():
    o = Mat4.orthographic(-4, 6, -1, 3, 0.5, 50)
    for point, expected in (((-4, -1, -0.5, 1), (-1, -1, -1)), ((6, 3, -50, 1), (1, 1, 1)),
                            ((1, 1, -25.25, 1), (0, 0, 0))):
        clip = o.multiplyVector4(Vec4(*point))
        assert clip.w == 1
        for got, want in zip((clip.x, clip.y, clip.z), expected):
            assert abs(got - want) <= 1e-9


def test_perspective_maps_near_and_far_to_depth_minus_one_and_one():
    near, far = 0.01, 1000.0
    p = Mat4.perspective(math.pi / 2.0, 1.5, near, far)
    for z_view, ndc in ((-near, -1.0), (-far, 1.0)):
        clip = p.multiplyVector4(Vec4(0, 0, z_view, 1))
        assert abs(clip.z / clip.w - ndc) <= 1e-9
        assert abs(clip.w + z_view) <= 1e-9  # w is the distance in front


def test_perspective_keeps_the_field_of_view_and_aspect():
    p = Mat4.perspective(math.pi / 2.0, 2.0, 0.1, 100.0)
    top = p.multiplyVector4(Vec4(0, 10, -10, 1))
    side = p.multiplyVector4(Vec4(20, 0, -10, 1))
    assert abs(top.y / top.w - 1.0) <= 1e-9
    assert abs(side.x / side.w - 1.0) <= 1e-9


def test_look_at_points_minus_z_at_the_target():
    eye, target = Vec3(3, 4, 12), Vec3(0, 1, 0)
    m = Mat4.lookAt(eye, target, Vec3(0, 1, 0))
    origin = m.multiplyVector4(Vec4(0, 0, 0, 1))
    assert (origin.x, origin.y, origin.z) == eye.tuple()
    forward = m.multiplyVector4(Vec4(0, 0, -1, 0))
    expected = target.subtract(eye).normalized()
    for got, want in zip((forward.x, forward.y, forward.z), expected.tuple()):
        assert abs(got - want) <= 1e-9
    assert m.multiplyVector4(Vec4(0, 1, 0, 0)).y > 0.0
    assert abs(m.multiplyVector4(Vec4(1, 0, 0, 0)).y) <= 1e-9  # right is level
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


def test_vec4_lerp_interpolates_every_component():
    assert Vec4(0, 10, -10, 1).lerp(Vec4(10, 20, 10, 3), 0.25).tuple() == (2.5, 12.5, -5, 1.5)
    assert Vec4(1, 2, 3, 4).dot(Vec4(1, 1, 1, 1)) == 10


def test_multiply_vector3_and_direction_agree_with_vector4():
    nxt = random(3)
    for _ in range(20):
        m = random_matrix(nxt)
        v = Vec3(nxt(), nxt(), nxt())
        point = m.multiplyVector4(Vec4(v.x, v.y, v.z, 1.0))
        direction = m.multiplyVector4(Vec4(v.x, v.y, v.z, 0.0))
        p, d = m.multiplyVector3(v), m.multiplyDirection(v)
        assert [f"{x:.6f}" for x in p.tuple()] == [f"{x:.6f}" for x in (point.x, point.y, point.z)]
        assert [f"{x:.6f}" for x in d.tuple()] == [f"{x:.6f}" for x in (direction.x, direction.y, direction.z)]


def test_transpose_swaps_rows_and_columns():
    m = rows([[1, 2, 3, 4], [5, 6, 7, 8], [9, 10, 11, 12], [13, 14, 15, 16]])
    t = m.transpose()
    for r in range(4):
        for c in range(4):
            assert t.value(r, c) == m.value(c, r)
