"""Minimal stand-in for numpy-quaternion: np.quaternion and rotate_vectors.

rotate_vectors applies the rotation matrix of q (divided by |q|^2, so q need
not be a unit quaternion) to each vector, in float64.
"""
import numpy as np


class quaternion:  # noqa: N801 - the library's own spelling
    __slots__ = ("w", "x", "y", "z")

    def __init__(self, w=0.0, x=0.0, y=0.0, z=0.0):
        self.w, self.x, self.y, self.z = float(w), float(x), float(y), float(z)

    @property
    def real(self):
        return self.w

    @property
    def imag(self):
        return np.array([self.x, self.y, self.z])

    def conj(self):
        return quaternion(self.w, -self.x, -self.y, -self.z)

    def __mul__(self, o):
        if not isinstance(o, quaternion):
            return quaternion(self.w * o, self.x * o, self.y * o, self.z * o)
        a1, b1, c1, d1 = self.w, self.x, self.y, self.z
        a2, b2, c2, d2 = o.w, o.x, o.y, o.z
        return quaternion(a1 * a2 - b1 * b2 - c1 * c2 - d1 * d2,
                          a1 * b2 + b1 * a2 + c1 * d2 - d1 * c2,
                          a1 * c2 - b1 * d2 + c1 * a2 + d1 * b2,
                          a1 * d2 + b1 * c2 - c1 * b2 + d1 * a2)

    def __repr__(self):
        return "quaternion(%r, %r, %r, %r)" % (self.w, self.x, self.y, self.z)


def as_rotation_matrix(q):
    w, x, y, z = q.w, q.x, q.y, q.z
    n = w * w + x * x + y * y + z * z
    return np.array([
        [1.0 - 2.0 * (y * y + z * z) / n, 2.0 * (x * y - z * w) / n, 2.0 * (x * z + y * w) / n],
        [2.0 * (x * y + z * w) / n, 1.0 - 2.0 * (x * x + z * z) / n, 2.0 * (y * z - x * w) / n],
        [2.0 * (x * z - y * w) / n, 2.0 * (y * z + x * w) / n, 1.0 - 2.0 * (x * x + y * y) / n],
    ])


def rotate_vectors(q, v):
    m = as_rotation_matrix(q)
    v = np.asarray(v, dtype=float)
    return np.einsum("ij,...j->...i", m, v)


np.quaternion = quaternion
