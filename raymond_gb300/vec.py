"""Vectors and 4×4 matrices of the public API (src/Vec2.mjs, src/Vec3.mjs,
src/Mat4.mjs), with the reference's operation order so packed values
(a box's inverse matrix, a camera basis) round identically."""

from __future__ import annotations

import math


class Vec2:
    __slots__ = ("x", "y")

    def __init__(self, x: float = 0.0, y: float = 0.0):
        self.x = float(x)
        self.y = float(y)

    def __repr__(self):
        return f"Vec2({self.x}, {self.y})"


class Vec3:
    """src/Vec3.mjs."""

    __slots__ = ("x", "y", "z")

    def __init__(self, x: float = 0.0, y: float = 0.0, z: float = 0.0):
        self.x = float(x)
        self.y = float(y)
        self.z = float(z)

    def add(self, o: "Vec3") -> "Vec3":
        return Vec3(self.x + o.x, self.y + o.y, self.z + o.z)

    def subtract(self, o: "Vec3") -> "Vec3":
        return Vec3(self.x - o.x, self.y - o.y, self.z - o.z)

    def scale(self, f: float) -> "Vec3":
        return Vec3(self.x * f, self.y * f, self.z * f)

    def multiply(self, o: "Vec3") -> "Vec3":
        return Vec3(self.x * o.x, self.y * o.y, self.z * o.z)

    def negate(self) -> "Vec3":
        return Vec3(-self.x, -self.y, -self.z)

    def lerp(self, o: "Vec3", t: float) -> "Vec3":
        return Vec3(self.x + (o.x - self.x) * t, self.y + (o.y - self.y) * t, self.z + (o.z - self.z) * t)

    def cross(self, o: "Vec3") -> "Vec3":
        return Vec3(self.y * o.z - self.z * o.y, self.z * o.x - self.x * o.z, self.x * o.y - self.y * o.x)

    def dot(self, o: "Vec3") -> float:
        return self.x * o.x + self.y * o.y + self.z * o.z

    def length(self) -> float:
        return math.sqrt(self.x * self.x + self.y * self.y + self.z * self.z)

    def normalized(self) -> "Vec3":
        n = self.length()
        return Vec3(self.x / n, self.y / n, self.z / n)

    def tuple(self):
        return (self.x, self.y, self.z)

    def __repr__(self):
        return f"Vec3({self.x}, {self.y}, {self.z})"


class Mat4:
    """Row-major 4×4 matrix acting on column vectors (src/Mat4.mjs)."""

    __slots__ = ("v",)

    def __init__(self, *values):
        if len(values) != 16:
            raise ValueError("A 4 x 4 matrix needs 16 values.")
        self.v = [float(x) for x in values]

    # Element indices run 0 to 3; the reference throws RangeError outside
    # that (src/Mat4.mjs:53-93, 396-400), the mirror raises ValueError.
    @staticmethod
    def _check(row: int, column: int):
        if not (0 <= row <= 3 and 0 <= column <= 3):
            raise ValueError(f"No element ({row}, {column}) in a 4 x 4 matrix.")

    def value(self, row: int, column: int) -> float:
        Mat4._check(row, column)
        return self.v[row * 4 + column]

    def setValue(self, row: int, column: int, value: float) -> None:
        Mat4._check(row, column)
        self.v[row * 4 + column] = float(value)

    @staticmethod
    def identity() -> "Mat4":
        return Mat4(1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)

    @staticmethod
    def translate(x, y, z) -> "Mat4":
        return Mat4(1, 0, 0, x, 0, 1, 0, y, 0, 0, 1, z, 0, 0, 0, 1)

    @staticmethod
    def scale(x, y, z) -> "Mat4":
        return Mat4(x, 0, 0, 0, 0, y, 0, 0, 0, 0, z, 0, 0, 0, 0, 1)

    @staticmethod
    def rotateX(theta) -> "Mat4":
        s, c = math.sin(theta), math.cos(theta)
        return Mat4(1, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1)

    @staticmethod
    def rotateY(theta) -> "Mat4":
        s, c = math.sin(theta), math.cos(theta)
        return Mat4(c, 0, s, 0, 0, 1, 0, 0, -s, 0, c, 0, 0, 0, 0, 1)

    @staticmethod
    def rotateZ(theta) -> "Mat4":
        s, c = math.sin(theta), math.cos(theta)
        return Mat4(c, -s, 0, 0, s, c, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)

    @staticmethod
    def lookAt(eye: Vec3, target: Vec3, up: Vec3) -> "Mat4":
        look = target.subtract(eye).normalized()
        right = look.cross(up).normalized()
        true_up = right.cross(look)
        return Mat4(right.x, true_up.x, -look.x, eye.x,
                    right.y, true_up.y, -look.y, eye.y,
                    right.z, true_up.z, -look.z, eye.z,
                    0, 0, 0, 1)

    def multiplyMat4(self, o: "Mat4") -> "Mat4":
        a, b = self.v, o.v
        out = [0.0] * 16
        for r in range(4):
            for c in range(4):
                out[r * 4 + c] = (a[r * 4] * b[c] + a[r * 4 + 1] * b[4 + c] + a[r * 4 + 2] * b[8 + c]
                                  + a[r * 4 + 3] * b[12 + c])
        return Mat4(*out)

    def multiplyVector3(self, p: Vec3) -> Vec3:
        m = self.v
        return Vec3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
                    m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
                    m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11])

    def multiplyDirection(self, p: Vec3) -> Vec3:
        m = self.v
        return Vec3(m[0] * p.x + m[1] * p.y + m[2] * p.z,
                    m[4] * p.x + m[5] * p.y + m[6] * p.z,
                    m[8] * p.x + m[9] * p.y + m[10] * p.z)

    def transpose(self) -> "Mat4":
        m = self.v
        return Mat4(*[m[c * 4 + r] for r in range(4) for c in range(4)])

    # Cofactor expansion along the first row, through 3×3 and 2×2 minors
    # (src/Mat4.mjs:96-130, src/Mat3.mjs:62-75, src/Mat2.mjs:30-33).
    @staticmethod
    def _det2(a):
        return a[0] * a[3] - a[1] * a[2]

    @staticmethod
    def _det3(a):
        det = 0.0
        for column in range(3):
            sub = [a[i * 3 + j] for i in range(1, 3) for j in range(3) if j != column]
            minor = Mat4._det2(sub)
            cof = -minor if column % 2 == 1 else minor
            det += a[column] * cof
        return det

    def _cofactor(self, row, column):
        sub = [self.v[i * 4 + j] for i in range(4) for j in range(4) if i != row and j != column]
        minor = Mat4._det3(sub)
        return -minor if (row + column) % 2 == 1 else minor

    def determinant(self) -> float:
        det = 0.0
        for column in range(4):
            det += self.v[column] * self._cofactor(0, column)
        return det

    def inverse(self) -> "Mat4":
        det = self.determinant()
        if det == 0.0:
            raise ValueError("The matrix has no inverse.")
        out = [0.0] * 16
        for row in range(4):
            for column in range(4):
                out[column * 4 + row] = self._cofactor(row, column) / det
        return Mat4(*out)
