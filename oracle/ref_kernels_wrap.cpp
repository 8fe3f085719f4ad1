// C entry points around the reference's own src/Kernels.cpp, compiled
// unmodified with -DDoublePrec against oracle/ref_shim (see oracle/Makefile).
// TEST INFRASTRUCTURE ONLY: used to pin the oracle's HavelockGF and Rankine
// point kernels against the reference's arithmetic.  The reference file is
// included from the reference tree at build time; nothing of it is copied.
#include "Kernels.cpp"

extern "C" {

// HavelockGF (Kernels.cpp:342-412) at n points -> 8 doubles each:
// Re/Im of G, dG/dx, dG/dy, dG/dz.
void ref_havelock(int n, const double* x, const double* y, const double* v, double* out) {
    for (int i = 0; i < n; ++i) {
        CReal G, DX, DY, DZ;
        BEMUse::HavelockGF(x[i], y[i], v[i], G, DX, DY, DZ);
        double* o = out + 8 * i;
        o[0] = G.real(); o[1] = G.imag(); o[2] = DX.real(); o[3] = DX.imag();
        o[4] = DY.real(); o[5] = DY.imag(); o[6] = DZ.real(); o[7] = DZ.imag();
    }
}

// Struve H0/H1 and the Bessel wrappers (Kernels.cpp:31-116) at n points.
void ref_special(int n, const double* x, double* out) {
    for (int i = 0; i < n; ++i) {
        double* o = out + 6 * i;
        o[0] = BEMUse::StruveH0(x[i]); o[1] = BEMUse::StruveH1(x[i]);
        o[2] = BEMUse::BesselJ0(x[i]); o[3] = BEMUse::BesselJ1(x[i]);
        o[4] = BEMUse::BesselY0(x[i]); o[5] = BEMUse::BesselY1(x[i]);
    }
}

// Source_Kernel / Dipole_Kernel (Kernels.cpp:11-27).
void ref_point_kernels(int n, const double* S, const double* D, const double* A, double* src, double* dip) {
    for (int i = 0; i < n; ++i) {
        Vector3 s(S[3 * i], S[3 * i + 1], S[3 * i + 2]);
        Vector3 d(D[3 * i], D[3 * i + 1], D[3 * i + 2]);
        Vector3 a(A[3 * i], A[3 * i + 1], A[3 * i + 2]);
        src[i] = BEMUse::Source_Kernel(s, d);
        dip[i] = BEMUse::Dipole_Kernel(s, d, a);
    }
}

}  // extern "C"
