"""The oracle's geometry from all nrdofH geometry dof (geom3D.F90:30-112),
pinned by a curved element with a closed-form map and volume.

On the unit cube, the quadratic dof of the two edges parallel to xi_1 at
xi_2 = 1 (edges 2 and 6: v2 -> v3 and v6 -> v7) carry a y-displacement.  The
quadratic edge function is -xi(1-xi) along its edge times the blending of the
other two coordinates, so the dof -c on both edges give the exact map

    x = xi_1,   y = xi_2 (1 + c xi_1 (1 - xi_1)),   z = xi_3,

with det J = 1 + c xi_1 (1 - xi_1) and volume 1 + c/6.  The vertex functions
sum to one, so with f = 1 the vertex entries of the element load sum to the
volume.  The element matrices on the same curved geometry are the GPU's
parity reference (tests/test_gpu_isoparametric.py).
"""
import numpy as np
import pytest

from oracle import oracle as O

CUBE = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                 [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=float)


def _curved_xnod(p, c):
    no = [p] * 12 + [11 * p] * 6 + [111 * p]
    n = O.nrdofH(1, no)
    x = np.zeros((n, 3))
    x[:8] = CUBE
    for edge in (2, 6):  # first (quadratic) function of the edge
        x[8 + edge * (p - 1), 1] = -c
    return no, x


@pytest.mark.parametrize("p", [2, 3, 4])
def test_curved_map_is_the_closed_form(p):
    c = 0.3
    no, xn = _curved_xnod(p, c)
    rng = np.random.default_rng(p)
    for xi in rng.uniform(0, 1, (20, 3)):
        v, g = O.shape_hexa(xi, no)
        X = v @ xn
        J = g.T @ xn  # J[c, i] = d x_i / d xi_c
        assert np.allclose(X, [xi[0], xi[1] * (1 + c * xi[0] * (1 - xi[0])), xi[2]], atol=1e-14)
        assert np.linalg.det(J) == pytest.approx(1 + c * xi[0] * (1 - xi[0]), abs=1e-13)


@pytest.mark.parametrize("p,integration", [(2, 0), (3, 0), (4, 1)])
def test_curved_element_volume(p, integration):
    c = 0.3
    no, xn = _curved_xnod(p, c)
    K, b, rc = O.elem(1, no, np.zeros(12), np.zeros(6), xn, 1.0, isol=11, integration=integration)
    assert rc == 0
    assert b[:8].sum() == pytest.approx(1 + c / 6, abs=1e-13)
    # the stiffness kills constants on any geometry
    assert np.abs(K @ np.r_[np.ones(8), np.zeros(K.shape[0] - 8)]).max() < 1e-12
