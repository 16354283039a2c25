// Plain-loop BLAS/LAPACK routines with the Fortran ABI that the reference's
// blas_lapack.h declares (zgetrf_, zgetri_, zgemv_, zgemm_, zgeru_,
// zdotu_sub_).  Used only to link the reference sources into the parity
// oracle (oracle/_ref); the reference's own BLAS is not vendored or pinned.
// Semantics follow the published reference BLAS/LAPACK definitions:
// column-major storage, partial pivoting on max |re|+|im| (izamax), unblocked
// LU (zgetf2) and inverse from the LU factors (zgetri).
#include <complex>
#include <cmath>
#include <vector>

typedef std::complex<double> zc;

static inline double cabs1(const zc& z) { return std::fabs(z.real()) + std::fabs(z.imag()); }

extern "C" void zgetrf_(const int* M, const int* N, double* Ad, const int* LDA, int* ipiv, int* info)
{
    zc* a = reinterpret_cast<zc*>(Ad);
    int m = *M, n = *N, lda = *LDA;
    *info = 0;
    int mn = m < n ? m : n;
    for (int j = 0; j < mn; ++j) {
        int p = j;
        double best = -1;
        for (int i = j; i < m; ++i) {
            double v = cabs1(a[i + (size_t)j * lda]);
            if (v > best) { best = v; p = i; }
        }
        ipiv[j] = p + 1;
        if (a[p + (size_t)j * lda] != zc(0, 0)) {
            if (p != j)
                for (int c = 0; c < n; ++c) std::swap(a[j + (size_t)c * lda], a[p + (size_t)c * lda]);
            zc r = zc(1, 0) / a[j + (size_t)j * lda];
            for (int i = j + 1; i < m; ++i) a[i + (size_t)j * lda] *= r;
        } else if (*info == 0) {
            *info = j + 1;
        }
        for (int c = j + 1; c < n; ++c) {
            zc t = a[j + (size_t)c * lda];
            if (t != zc(0, 0))
                for (int i = j + 1; i < m; ++i) a[i + (size_t)c * lda] -= a[i + (size_t)j * lda] * t;
        }
    }
}

extern "C" void zgetri_(const int* N, double* Ad, const int* LDA, const int* ipiv, double* workd,
                        const int* lwork, int* info)
{
    (void)workd; (void)lwork;
    zc* a = reinterpret_cast<zc*>(Ad);
    int n = *N, lda = *LDA;
    *info = 0;
    std::vector<zc> work(n);
    for (int j = 0; j < n; ++j) {            // inv(U), ztrti2
        a[j + (size_t)j * lda] = zc(1, 0) / a[j + (size_t)j * lda];
        zc ajj = -a[j + (size_t)j * lda];
        for (int k = 0; k < j; ++k) {
            zc t = a[k + (size_t)j * lda];
            if (t != zc(0, 0)) {
                for (int i = 0; i < k; ++i) a[i + (size_t)j * lda] += t * a[i + (size_t)k * lda];
                a[k + (size_t)j * lda] = t * a[k + (size_t)k * lda];
            }
        }
        for (int i = 0; i < j; ++i) a[i + (size_t)j * lda] *= ajj;
    }
    for (int j = n - 1; j >= 0; --j) {        // solve inv(A)*L = inv(U)
        for (int i = j + 1; i < n; ++i) { work[i] = a[i + (size_t)j * lda]; a[i + (size_t)j * lda] = 0; }
        for (int c = j + 1; c < n; ++c) {
            zc t = work[c];
            for (int i = 0; i < n; ++i) a[i + (size_t)j * lda] -= a[i + (size_t)c * lda] * t;
        }
    }
    for (int j = n - 2; j >= 0; --j) {
        int jp = ipiv[j] - 1;
        if (jp != j)
            for (int i = 0; i < n; ++i) std::swap(a[i + (size_t)j * lda], a[i + (size_t)jp * lda]);
    }
}

extern "C" void zgemv_(const char* trans, const int* M, const int* N, const double* alphad,
                       const double* Ad, const int* lda, const double* xd, const int* incx,
                       const double* betad, double* yd, const int* incy)
{
    const zc* a = reinterpret_cast<const zc*>(Ad);
    const zc* x = reinterpret_cast<const zc*>(xd);
    zc* y = reinterpret_cast<zc*>(yd);
    zc alpha = *reinterpret_cast<const zc*>(alphad), beta = *reinterpret_cast<const zc*>(betad);
    int m = *M, n = *N;
    bool nt = (*trans == 'N' || *trans == 'n');
    int leny = nt ? m : n, lenx = nt ? n : m;
    for (int i = 0; i < leny; ++i) {
        zc& yi = y[(size_t)i * *incy];
        yi = (beta == zc(0, 0)) ? zc(0, 0) : beta * yi;
    }
    if (nt) {
        for (int j = 0; j < lenx; ++j) {
            zc t = alpha * x[(size_t)j * *incx];
            for (int i = 0; i < m; ++i) y[(size_t)i * *incy] += t * a[i + (size_t)j * *lda];
        }
    } else {
        for (int j = 0; j < n; ++j) {
            zc s = 0;
            for (int i = 0; i < m; ++i) s += a[i + (size_t)j * *lda] * x[(size_t)i * *incx];
            y[(size_t)j * *incy] += alpha * s;
        }
    }
}

extern "C" void zgemm_(const char* ta, const char* tb, const int* M, const int* N, const int* K,
                       const double* alphad, const double* Ad, const int* lda, const double* Bd,
                       const int* ldb, const double* betad, double* Cd, const int* ldc)
{
    (void)ta; (void)tb;   // the reference calls only 'N','N'
    const zc* a = reinterpret_cast<const zc*>(Ad);
    const zc* b = reinterpret_cast<const zc*>(Bd);
    zc* c = reinterpret_cast<zc*>(Cd);
    zc alpha = *reinterpret_cast<const zc*>(alphad), beta = *reinterpret_cast<const zc*>(betad);
    int m = *M, n = *N, k = *K;
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < m; ++i) {
            zc& cij = c[i + (size_t)j * *ldc];
            cij = (beta == zc(0, 0)) ? zc(0, 0) : beta * cij;
        }
        for (int l = 0; l < k; ++l) {
            zc t = alpha * b[l + (size_t)j * *ldb];
            for (int i = 0; i < m; ++i) c[i + (size_t)j * *ldc] += t * a[i + (size_t)l * *lda];
        }
    }
}

extern "C" void zgeru_(const int* M, const int* N, const double* alphad, const double* xd,
                       const int* incx, const double* yd, const int* incy, double* Ad, const int* lda)
{
    const zc* x = reinterpret_cast<const zc*>(xd);
    const zc* y = reinterpret_cast<const zc*>(yd);
    zc* a = reinterpret_cast<zc*>(Ad);
    zc alpha = *reinterpret_cast<const zc*>(alphad);
    for (int j = 0; j < *N; ++j) {
        zc t = alpha * y[(size_t)j * *incy];
        for (int i = 0; i < *M; ++i) a[i + (size_t)j * *lda] += x[(size_t)i * *incx] * t;
    }
}

extern "C" void zdotu_sub_(const int* N, const double* xd, const int* incx, const double* yd,
                           const int* incy, double* out)
{
    const zc* x = reinterpret_cast<const zc*>(xd);
    const zc* y = reinterpret_cast<const zc*>(yd);
    zc s = 0;
    for (int i = 0; i < *N; ++i) s += x[(size_t)i * *incx] * y[(size_t)i * *incy];
    *reinterpret_cast<zc*>(out) = s;
}
