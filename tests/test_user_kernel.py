"""User kernels compiled at run time (hmgpu_user_kernel_compile), on the CPU:
the entry function compiles with NVRTC into the library's entry kernels, and a
source that does not compile is refused with the compiler's log, line numbers
counted from the user's own first line."""
import pytest

import hmgpu

LAPLACE = """__device__ double hmgpu_entry(const double *x, const double *y, const double *p, int a, int b) {
  double dx = x[0] - y[0], dy = x[1] - y[1], dz = x[2] - y[2];
  double r = sqrt(dx * dx + dy * dy + dz * dz);
  return r == 0.0 ? 0.0 : 0.07957747154594767 / r;
}
"""


def test_compiles_and_frees():
    uk = hmgpu.UserKernel(LAPLACE)
    assert uk._h.value
    K = hmgpu.Kernel("user", [[0.0, 1.0], [0.0, 0.0], [0.0, 0.0]], user=uk, params=[2.0, 3.0])
    d = K.desc()
    assert d.kind == 6 and d.nparams == 2 and d.user == uk._h.value and d.nX == 2
    del K, d
    del uk


def test_compile_error_reports_the_users_line():
    bad = "__device__ double hmgpu_entry(const double *x, const double *y, const double *p, int a, int b) {\n" \
          "  return x[0] +* y[0];\n}\n"
    with pytest.raises(hmgpu.HMGPUError) as e:
        hmgpu.UserKernel(bad)
    assert e.value.code == -1
    assert "user_kernel.cu(2): error" in e.value.log, e.value.log


def test_source_without_the_entry_function_is_refused():
    with pytest.raises(hmgpu.HMGPUError, match="hmgpu_entry"):
        hmgpu.UserKernel("__device__ double f(double a) { return a; }")


def test_kernel_needs_a_user_function():
    with pytest.raises(ValueError):
        hmgpu.Kernel("user", [[0.0], [0.0], [0.0]])
