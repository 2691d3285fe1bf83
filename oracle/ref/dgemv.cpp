// Naive column-major dgemv_ (BLAS level 2): y = alpha*op(A)*x + beta*y.
// The reference calls it from Poisson/DFTPatchSolver.h:249-261; no BLAS is
// installed here, so this plain loop (summing j in increasing order) stands
// in for it.  The oracle restatement sums in the same order.
// TEST INFRASTRUCTURE ONLY.
extern "C" void dgemv_(char& t, int& m, int& n, double& alpha, double* A, int& lda, double* x,
                       int& incx, double& beta, double* y, int& incy) {
  bool tr = (t == 'T' || t == 't');
  int ylen = tr ? n : m, xlen = tr ? m : n;
  for (int i = 0; i < ylen; i++) {
    double s = 0;
    for (int j = 0; j < xlen; j++) {
      double a = tr ? A[j + (long)i * lda] : A[i + (long)j * lda];
      s += a * x[(long)j * incx];
    }
    y[(long)i * incy] = alpha * s + (beta == 0 ? 0 : beta * y[(long)i * incy]);
  }
}
