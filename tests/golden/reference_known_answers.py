"""Known answers transcribed from the reference's own tests (luiswirth/formoniq),
each with the file:line it comes from. These pin the oracle; the GPU path is then
checked against the oracle.

The reference is Rust and cannot be executed here, so its tests' literal
expected values are the golden vectors.
"""
import numpy as np

# crates/formoniq/src/operators.rs:931-943 (hodge_mass_dim2_grade1): the grade-1
# Hodge mass on the unit triangle.
HODGE_MASS_DIM2_GRADE1 = np.array([
    [1 / 3, 1 / 6, 0.0],
    [1 / 6, 1 / 3, 0.0],
    [0.0, 0.0, 1 / 6],
])

# crates/formoniq/src/operators.rs:945-959 (dif_trial_n2_k1)
DIF_TRIAL_N2_K1 = np.array([
    [-1 / 2, 1 / 3, 1 / 6],
    [-1 / 2, 1 / 6, 1 / 3],
    [0.0, -1 / 6, 1 / 6],
])

# crates/formoniq/src/operators.rs:961-975 (dif_test_n2_k1)
DIF_TEST_N2_K1 = np.array([
    [-1 / 2, -1 / 2, 0.0],
    [1 / 3, 1 / 6, -1 / 6],
    [1 / 6, 1 / 3, 1 / 6],
])

# crates/formoniq/tests/unit_elmat.rs:59-84 (unit_mass): grade-0 mass on the unit
# simplex for dims 0..3.
UNIT_MASS = {
    0: np.array([[1.0]]),
    1: np.array([[1 / 3, 1 / 6], [1 / 6, 1 / 3]]),
    2: np.array([[1 / 12, 1 / 24, 1 / 24], [1 / 24, 1 / 12, 1 / 24], [1 / 24, 1 / 24, 1 / 12]]),
    3: np.array([[1 / 60, 1 / 120, 1 / 120, 1 / 120], [1 / 120, 1 / 60, 1 / 120, 1 / 120],
                 [1 / 120, 1 / 120, 1 / 60, 1 / 120], [1 / 120, 1 / 120, 1 / 120, 1 / 60]]),
}


# crates/formoniq/tests/unit_elmat.rs:36-49 (unit_laplacian): dif_both(dim, 1) on
# the unit simplex, any dim: [0,0] = dim, [i,0] = [0,i] = -1, [i,i] = 1, times 1/dim!.
def unit_laplacian(dim: int) -> np.ndarray:
    import math
    n = dim + 1
    m = np.zeros((n, n))
    m[0, 0] = dim
    for i in range(1, n):
        m[i, 0] = m[0, i] = -1
        m[i, i] = 1
    return m / math.factorial(dim)


# crates/regge/src/mesher/cartesian.rs:243-271 (unit_cube_mesh): 3D, 1 box.
UNIT_CUBE_COORDS = np.array([
    [0., 0., 0.], [1., 0., 0.], [0., 1., 0.], [1., 1., 0.],
    [0., 0., 1.], [1., 0., 1.], [0., 1., 1.], [1., 1., 1.],
])
UNIT_CUBE_CELLS = np.array([
    [0, 1, 3, 7], [0, 2, 3, 7], [0, 1, 5, 7], [0, 4, 5, 7], [0, 2, 6, 7], [0, 4, 6, 7],
])

# crates/regge/src/mesher/cartesian.rs:273-300 (unit_square_mesh): 2D, 2 boxes.
UNIT_SQUARE_COORDS = np.array([
    [0.0, 0.0], [0.5, 0.0], [1.0, 0.0], [0.0, 0.5], [0.5, 0.5], [1.0, 0.5], [0.0, 1.0], [0.5, 1.0], [1.0, 1.0],
])
UNIT_SQUARE_CELLS = np.array([
    [0, 1, 4], [0, 3, 4], [1, 2, 5], [1, 4, 5], [3, 4, 7], [3, 6, 7], [4, 5, 8], [4, 7, 8],
])

# crates/simplicial/src/mesher/grid.rs:124-140: Kuhn cells of cube(3, 1), colex.
KUHN_CUBE3_CELLS = UNIT_CUBE_CELLS

# crates/formoniq/tests/fdm.rs:103-127 (LAPLACE_MATRICES_INTERIOR): the FDM
# Laplacian on 1..3 interior vertices per axis, dims 1..3 (index = dim).
LAPLACE_MATRICES_INTERIOR = {
    1: np.array([[2, -1], [-1, 2]]),
    2: np.array([[4, -1, -1, 0], [-1, 4, 0, -1], [-1, 0, 4, -1], [0, -1, -1, 4]]),
    3: np.array([
        [6, -1, -1, 0, -1, 0, 0, 0], [-1, 6, 0, -1, 0, -1, 0, 0], [-1, 0, 6, -1, 0, 0, -1, 0],
        [0, -1, -1, 6, 0, 0, 0, -1], [-1, 0, 0, 0, 6, -1, -1, 0], [0, -1, 0, 0, -1, 6, 0, -1],
        [0, 0, -1, 0, -1, 0, 6, -1], [0, 0, 0, -1, 0, -1, -1, 6],
    ]),
}

# crates/formoniq/tests/fem3d.rs:34-41: the six Kuhn tets of a box, in the
# reference's hand-written FEM (local vertex ids i + 2j + 4k).
FEM3D_TETS = [[0, 1, 3, 7], [0, 1, 5, 7], [0, 2, 3, 7], [0, 2, 6, 7], [0, 4, 5, 7], [0, 4, 6, 7]]

# crates/formoniq/src/problems/elliptic.rs:280-284: block-MINRES vs LU on the
# mixed system agrees to 1e-7 (dims 1..3, N = 2, relative complex, rtol 1e-11).
BLOCK_MINRES_VS_LU_TOL = 1e-7
# crates/formoniq/src/problems/elliptic.rs:362-366: iteration growth bound.
MINRES_ITER_SLACK = 8
