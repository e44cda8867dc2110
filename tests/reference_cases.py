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


# ---------------------------------------------------- bicg / cgs / qmr / minres / lgmres
# tests/linalg_new_tests.rs:34-79 -- bicg on [[2,-1],[1,3]], b = [3, 2] -> [11/7, 1/7] (1e-5)
BICG_2X2 = dict(rows=[0, 0, 1, 1], cols=[0, 1, 0, 1], data=[2.0, -1.0, 1.0, 3.0], shape=(2, 2),
                b=[3.0, 2.0], atol=1e-8, rtol=1e-8, x=[11.0 / 7.0, 1.0 / 7.0], tol=1e-5, resid=1e-5)

# tests/cgs_revised_tests.rs:6-26 -- identity: converged in exactly 1 iteration
CGS_IDENTITY = dict(rows=[0, 1, 2], cols=[0, 1, 2], data=[1.0, 1.0, 1.0], shape=(3, 3), b=[1.0, 2.0, 3.0],
                    iterations=1, tol=1e-10)
# tests/cgs_revised_tests.rs:28-61 -- diagonally dominant non-symmetric 3x3, true residual < 1e-8
CGS_WELL = dict(rows=[0, 0, 0, 1, 1, 1, 2, 2, 2], cols=[0, 1, 2, 0, 1, 2, 0, 1, 2],
                data=[4.0, 0.5, 0.5, 0.5, 4.0, 0.5, 0.0, 0.5, 4.0], shape=(3, 3), b=[5.0, 5.0, 4.5],
                rtol=1e-8, atol=1e-10, resid=1e-8)
# tests/cgs_revised_tests.rs:63-108 -- 4x4 with / without right Jacobi (rtol 1e-6, 100 its)
CGS_PRECOND = dict(rows=[r for r in range(4) for _ in range(4)], cols=[c for _ in range(4) for c in range(4)],
                   data=[10.0, 1.0, 0.5, 0.0, 1.0, 8.0, 0.5, 0.5, 0.5, 0.5, 6.0, 1.0, 0.0, 0.5, 1.0, 4.0],
                   shape=(4, 4), b=[11.5, 10.0, 8.0, 5.5], max_iter=100, rtol=1e-6)
# tests/cgs_revised_tests.rs:182-209 -- SPD 3x3: converged, x = [1, 1, 1] (1e-6)
CGS_SPD = dict(rows=[0, 0, 0, 1, 1, 1, 2, 2, 2], cols=[0, 1, 2, 0, 1, 2, 0, 1, 2],
               data=[4.0, -1.0, -1.0, -1.0, 4.0, -1.0, -1.0, -1.0, 4.0], shape=(3, 3), b=[2.0, 2.0, 2.0],
               rtol=1e-8, x=[1.0, 1.0, 1.0], tol=1e-6)


# tests/cgs_revised_tests.rs:110-180 -- 5x5-grid Laplacian (25 x 25), b = 1..25,
# max_iter 200, rtol 1e-5, atol 1e-7: if converged, relative true residual < 1e-4
def cgs_laplacian(n=5):
    rows, cols, data = [], [], []
    for i in range(n):
        for j in range(n):
            idx = i * n + j
            rows.append(idx); cols.append(idx); data.append(4.0)
            if i > 0:
                rows.append(idx); cols.append((i - 1) * n + j); data.append(-1.0)
            if i < n - 1:
                rows.append(idx); cols.append((i + 1) * n + j); data.append(-1.0)
            if j > 0:
                rows.append(idx); cols.append(i * n + (j - 1)); data.append(-1.0)
            if j < n - 1:
                rows.append(idx); cols.append(i * n + (j + 1)); data.append(-1.0)
    return dict(rows=rows, cols=cols, data=data, shape=(n * n, n * n), b=[float(i + 1) for i in range(n * n)],
                max_iter=200, rtol=1e-5, atol=1e-7, rel=1e-4)


# qmr.rs:298-382 -- identity (1 iteration), diagonal, initial guess, max iterations
QMR_IDENTITY = dict(b=[1.0, 2.0, 3.0], iterations=1, tol=1e-10)
QMR_DIAG = dict(diag=[2.0, 3.0, 4.0], b=[2.0, 6.0, 8.0], x=[1.0, 2.0, 2.0], rtol=1e-10, atol=1e-12,
                max_iterations=10, tol=1e-9)
QMR_GUESS = dict(b=[1.0, 2.0, 3.0], x0=[0.9, 1.9, 2.9], rtol=1e-10, atol=1e-12, max_iterations=1, tol=1e-10)
QMR_MAXIT = dict(diag=[1e-8, 1.0, 1.0], b=[1.0, 1.0, 1.0], max_iter=5, rtol=1e-10, atol=1e-12)

# minres.rs:287-401 -- identity, indefinite diagonal, symmetric 3x3, Jacobi-like diagonal M
MINRES_IDENTITY = dict(b=[1.0, 2.0, 3.0], tol=1e-10)
MINRES_DIAG = dict(diag=[2.0, -3.0, 4.0], b=[2.0, -6.0, 12.0], x=[1.0, 2.0, 3.0], tol=1e-9)
MINRES_SYM = dict(rows=[0, 0, 1, 1, 1, 2, 2], cols=[0, 1, 0, 1, 2, 1, 2],
                  data=[4.0, -1.0, -1.0, 2.0, -1.0, -1.0, 4.0], shape=(3, 3), b=[1.0, 0.0, 1.0], tol=1e-9)
MINRES_PREC = dict(rows=[0, 0, 1, 1, 1, 2, 2], cols=[0, 1, 0, 1, 2, 1, 2],
                   data=[4.0, -1.0, -1.0, 4.0, -1.0, -1.0, 4.0], shape=(3, 3), b=[1.0, 2.0, 3.0],
                   prec=[0.25, 0.25, 0.25], tol=1e-9)

# lgmres.rs:335-366 -- identity (x = b, 1e-10) and from_raw_csr SPD (residual < 1e-8)
LGMRES_IDENTITY = dict(b=[1.0, 2.0, 3.0], tol=1e-10)
LGMRES_SPD = dict(data=[4.0, -1.0, -1.0, 4.0, -1.0, -1.0, 4.0], indptr=[0, 2, 5, 7],
                  indices=[0, 1, 0, 1, 2, 1, 2], b=[1.0, 2.0, 3.0], resid=1e-8)
