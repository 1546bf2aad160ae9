//
// Hand-written PTX with numba's device-function ABI, the one the reference
// links (int integrand(double* ret, double* x)): *ret = x0^2 + x1^2 + x2^2,
// evaluated as fma(x2, x2, fma(x1, x1, x0 * x0)).  Its integral over [0,1]^3 is 1.
//
.version 9.0
.target sm_103a
.address_size 64

.visible .func (.param .b32 func_retval0) integrand(
    .param .b64 integrand_param_0,
    .param .b64 integrand_param_1
)
{
    .reg .b32 %r<2>;
    .reg .b64 %rd<3>;
    .reg .f64 %fd<7>;

    ld.param.u64 %rd1, [integrand_param_0];
    ld.param.u64 %rd2, [integrand_param_1];
    ld.f64 %fd1, [%rd2];
    ld.f64 %fd2, [%rd2+8];
    ld.f64 %fd3, [%rd2+16];
    mul.rn.f64 %fd4, %fd1, %fd1;
    fma.rn.f64 %fd5, %fd2, %fd2, %fd4;
    fma.rn.f64 %fd6, %fd3, %fd3, %fd5;
    st.f64 [%rd1], %fd6;
    mov.u32 %r1, 0;
    st.param.b32 [func_retval0], %r1;
    ret;
}
