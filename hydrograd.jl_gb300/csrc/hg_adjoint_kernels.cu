// adjoint kernels (placeholder)
