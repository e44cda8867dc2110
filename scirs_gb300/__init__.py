"""GB300-native backend for the scirs2-sparse iterative-solve path.

CSR construction / transpose / SpMV, the LinearOperator slot (operators and
preconditioners), and the cg / bicgstab / gmres solvers run as hand-written
sm_103a CUDA kernels behind the C ABI in include/scirs_sparse.h; this
package is the Python mirror of the reference API over that ABI.
"""
from .sparse import (  # noqa: F401
    BatchedResult,
    Context,
    batched_pcg,
    generate_batch,
    IRResult,
    IterationResult,
    LearnedSAI,
    Operator,
    SparseError,
    bicgstab,
    cg,
    cg_mixed,
    spmv_kernel,
    sum_operator,
    product_operator,
    zero_operator,
    csr_array,
    csr_array_from_triplets,
    csr_from_arrays,
    csr_matrix,
    csr_matrix_from_raw,
    diagonal,
    fsai,
    generate,
    gmres,
    host_operator,
    ic0,
    identity,
    jacobi,
    jacobi_from_diagonal,
    message_string,
    rhs_normal,
    scaled_identity,
    true_rel_residual,
)
