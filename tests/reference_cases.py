"""The reference crate's own tests for the solve path, as data.

Each case cites the scirs2-sparse test it transcribes (inputs and the
expected values or properties the reference asserts).  Both the CPU oracle
(test_oracle_reference.py) and the device library (test_device_reference.py)
replay them.
"""
import numpy as np

# csr.rs:505-591 -- CsrMatrix::new, to_dense, dot, transpose
CSR_BASIC = dict(
    rows=[0, 0, 1, 2, 2], cols=[0, 2, 2, 0, 1], data=[1.0, 2.0, 3.0, 4.0, 5.0], shape=(3, 3),
    dense=[[1, 0, 2], [0, 0, 3], [4, 5, 0]],
    dot_x=[1.0, 2.0, 3.0], dot_y=[7.0, 9.0, 14.0],
    dense_t=[[1, 0, 4], [0, 0, 5], [2, 3, 0]],
)

# csr_array.rs:999-1076 -- CsrArray::new / from_triplets / dot_vector
CSR_ARRAY = dict(
    data=[1.0, 2.0, 3.0, 4.0, 5.0], indices=[0, 2, 1, 0, 2], indptr=[0, 2, 3, 5], shape=(3, 3),
    rows=[0, 0, 1, 2, 2], cols=[0, 2, 1, 0, 2],
    gets=[((0, 0), 1.0), ((0, 2), 2.0), ((1, 1), 3.0), ((2, 0), 4.0), ((2, 2), 5.0), ((0, 1), 0.0)],
    dot_x=[1.0, 2.0, 3.0], dot_y=[7.0, 6.0, 19.0],
)

# iterative.rs:870-892 (cg) and :923-944 (bicgstab, non-symmetric)
SPD3 = dict(rows=[0, 0, 0, 1, 1, 1, 2, 2, 2], cols=[0, 1, 2, 0, 1, 2, 0, 1, 2],
            data=[4.0, -1.0, -1.0, -1.0, 4.0, -1.0, -1.0, -1.0, 4.0], b=[1.0, 2.0, 3.0], tol=1e-9)
NONSYM3 = dict(rows=[0, 0, 0, 1, 1, 1, 2, 2, 2], cols=[0, 1, 2, 0, 1, 2, 0, 1, 2],
               data=[4.0, -1.0, -2.0, -1.0, 4.0, -1.0, 0.0, -1.0, 3.0], b=[1.0, 2.0, 1.0], tol=1e-9)

# tests/linalg_new_tests.rs:5-32 -- cg on [[2,-1],[-1,2]] -> [2/3, 1/3] (1e-6)
CG_2X2 = dict(rows=[0, 0, 1, 1], cols=[0, 1, 0, 1], data=[2.0, -1.0, -1.0, 2.0], b=[1.0, 0.0],
              x=[2.0 / 3.0, 1.0 / 3.0], tol=1e-6)

# tests/preconditioner_tests.rs:7-42 -- cg + Jacobi on tridiag(-1, 4, -1)
CG_JACOBI = dict(rows=[0, 0, 1, 1, 1, 2, 2], cols=[0, 1, 0, 1, 2, 1, 2],
                 data=[4.0, -1.0, -1.0, 4.0, -1.0, -1.0, 4.0], b=[2.0, 1.0, 2.0],
                 max_iterations=20, tol=1e-5)

# tests/preconditioner_tests.rs:44-63 and preconditioners.rs:405-419 -- Jacobi apply
JACOBI_APPLY = dict(diag=[2.0, 3.0, 4.0], x=[2.0, 6.0, 12.0], y=[1.0, 2.0, 3.0])

# iterative.rs:842-868, :894-921 -- identity and diagonal operators
IDENTITY_B = [1.0, 2.0, 3.0]
DIAG = dict(diag=[2.0, 3.0, 4.0], b=[2.0, 6.0, 12.0], x=[1.0, 2.0, 3.0])

# tests/bicgstab_tests.rs:6-53 -- duplicate (3,3) entry, left Jacobi
BICGSTAB_DUP = dict(rows=[0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 3], cols=[0, 1, 0, 1, 2, 1, 2, 3, 0, 2, 3, 3],
                    data=[10.0, 1.0, 2.0, 12.0, 1.0, 1.0, 8.0, 2.0, 3.0, 1.0, 15.0, 1.0],
                    shape=(4, 4), b=[11.0, 15.0, 11.0, 20.0], max_iter=100, rtol=1e-6, atol=1e-8,
                    max_iterations=50, resid=1e-6)


# tests/bicgstab_tests.rs:55-113 -- convection-diffusion n = 10
def convection_diffusion(n=10):
    rows, cols, data = [], [], []
    for i in range(n):
        rows.append(i); cols.append(i); data.append(4.0)
        if i > 0:
            rows.append(i); cols.append(i - 1); data.append(-1.5)
            rows.append(i - 1); cols.append(i); data.append(-0.5)
    b = [1.0 + i for i in range(n)]
    return dict(rows=rows, cols=cols, data=data, shape=(n, n), b=b, max_iter=200, rtol=1e-8,
                atol=1e-10, resid=5e-7)


# tests/bicgstab_tests.rs:115-137 -- singular system, breakdown reported
SINGULAR = dict(rows=[0, 0, 1, 1], cols=[0, 1, 0, 1], data=[1.0, 1.0, 1.0, 1.0], shape=(2, 2),
                b=[1.0, 2.0])

# ic.rs:237-255 (finite output) and :257-271 (non-SPD -> error)
IC0_SPD = dict(data=[4.0, -1.0, -1.0, 4.0, -1.0, -1.0, 4.0], indptr=[0, 2, 5, 7],
               indices=[0, 1, 0, 1, 2, 1, 2], b=[1.0, 2.0, 3.0])
IC0_NOT_SPD = dict(data=[1.0, 2.0, 3.0, 4.0], indptr=[0, 2, 4], indices=[0, 1, 0, 1])


def dense_of(rows, cols, data, shape):
    d = np.zeros(shape)
    for r, c, v in zip(rows, cols, data):
        d[r, c] += v
    return d
