// ratapprox.cu -- the rational approximations r(x) = a0 + sum_i a_i / (x + b_i)
// of the RHMC (src/RationalApprox/rationalapprox.c): the .REMEZ text files,
// their rescaling to the spectral range of M^+M, and evaluation.  Host code
// only; the shifts b_i and residues a_i feed multishift_invert, the batched
// multi-shift solver and the force.
//
// Every function is a weak symbol: a host program that still links the
// reference's own rationalapprox.c keeps its definitions, one that does not
// gets these.  Names, arguments, file format, messages and failure behaviour
// (exit on a malformed file or an uncovered range) follow the reference.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "../../include/ostaple_gb300.h"

extern "C" {

// approx_<num>_over_<den>_order_<n>_mloglm_<-log10 lambda_min>.REMEZ (rationalapprox.c:16-42)
__attribute__((weak)) char* rational_approx_filename_old(int approx_order, int exponent_num, int exponent_den,
                                                         double lambda_min) {
  char* name = static_cast<char*>(malloc(64));
  snprintf(name, 64, "approx_%d_over_%d_order_%d_mloglm_%1.1f.REMEZ", exponent_num, exponent_den, approx_order,
           -log(lambda_min) / log(10.0));
  return name;
}

// approx_<num>_over_<den>_mlogerr_<-log10 error>_mloglm_<-log10 lambda_min>.REMEZ (rationalapprox.c:44-70)
__attribute__((weak)) char* rational_approx_filename(double error, int exponent_num, int exponent_den,
                                                     double lambda_min) {
  char* name = static_cast<char*>(malloc(64));
  snprintf(name, 64, "approx_%d_over_%d_mlogerr_%1.1f_mloglm_%1.1f.REMEZ", exponent_num, exponent_den,
           -log(error) / log(10.0), -log(lambda_min) / log(10.0));
  return name;
}

// Reads a .REMEZ file (rationalapprox.c:83-117).  Returns 1 if the file does
// not exist; a file that does not have the expected entries ends the
// program, as in the reference.
__attribute__((weak)) int rationalapprox_read_custom_nomefile(RationalApprox* ra, char* nomefile) {
  FILE* f = fopen(nomefile, "rt");
  printf("%s\n", nomefile);
  if (!f) {
    printf("Rational Approximation File %s not found!\n", nomefile);
    return 1;
  }
  auto expect = [&](int got, int want, int line) {
    if (got != want) {
      printf("%s:%d, Error, not read expected number of entries : %d read vs %d should_read\n.", __FILE__, line, got,
             want);
      exit(1);
    }
  };
  expect(fscanf(f, "\nApproximation to f(x) = (x)^(%i/%i)\n", &ra->exponent_num, &ra->exponent_den), 2, __LINE__);
  expect(fscanf(f, "Order: %i\n", &ra->approx_order), 1, __LINE__);
  if (ra->approx_order < 0 || ra->approx_order > MAX_APPROX_ORDER) {
    printf("%s:%d, Error, approximation order %d outside [0, %d]\n", __FILE__, __LINE__, ra->approx_order,
           MAX_APPROX_ORDER);
    exit(1);
  }
  expect(fscanf(f, "Lambda Min: %lf\n", &ra->lambda_min), 1, __LINE__);
  expect(fscanf(f, "Lambda Max: %lf\n", &ra->lambda_max), 1, __LINE__);
  expect(fscanf(f, "GMP Remez Precision: %i\n", &ra->gmp_remez_precision), 1, __LINE__);
  expect(fscanf(f, "Error: %lf\n", &ra->error), 1, __LINE__);
  expect(fscanf(f, "RA_a0 = %lf\n", &ra->RA_a0), 1, __LINE__);
  for (int i = 0; i < ra->approx_order; ++i) {
    int ia = 0, ib = 0;
    expect(fscanf(f, "RA_a[%i] = %lf, RA_b[%i] = %lf\n", &ia, &ra->RA_a[i], &ib, &ra->RA_b[i]), 4, __LINE__);
  }
  fclose(f);
  return 0;
}

__attribute__((weak)) int rationalapprox_read(RationalApprox* ra) {
  char* name = rational_approx_filename(ra->error, ra->exponent_num, ra->exponent_den, ra->lambda_min);
  const int err = rationalapprox_read_custom_nomefile(ra, name);
  free(name);
  return err;
}

// Writes the .REMEZ format read above (rationalapprox.c:119-143).
__attribute__((weak)) void rationalapprox_save(const char* nomefile, RationalApprox* ra) {
  FILE* f = fopen(nomefile, "w");
  printf("%s\n", nomefile);
  if (!f) {
    printf("Could not open file %s \n", nomefile);
    exit(-1);
  }
  fprintf(f, "\nApproximation to f(x) = (x)^(%i/%i)\n", ra->exponent_num, ra->exponent_den);
  fprintf(f, "Order: %i\n", ra->approx_order);
  fprintf(f, "Lambda Min: %18.16e\n", ra->lambda_min);
  fprintf(f, "Lambda Max: %18.16e\n", ra->lambda_max);
  fprintf(f, "GMP Remez Precision: %i\n", ra->gmp_remez_precision);
  fprintf(f, "Error: %18.16e\n", ra->error);
  fprintf(f, "RA_a0 = %18.16e\n", ra->RA_a0);
  for (int i = 0; i < ra->approx_order; ++i)
    fprintf(f, "RA_a[%d] = %18.16e, RA_b[%d] = %18.16e\n", i, ra->RA_a[i], i, ra->RA_b[i]);
  fclose(f);
}

// A mother approximation on [lambda_min, 1] mapped to [0.95 min, 1.05 max]
// of the measured spectrum: x -> x / M with M = 1.05 max scales the shifts
// by M and the residues by M^(1 + p), a0 by M^p, p = num/den
// (rationalapprox.c:145-194).  Ends the program when the mapped range does
// not reach down to minmax[0]; warns when it reaches far below it.
__attribute__((weak)) void rescale_rational_approximation(RationalApprox* in, RationalApprox* out, double* minmax) {
  const double power = double(in->exponent_num) / in->exponent_den;
  out->exponent_num = in->exponent_num;
  out->exponent_den = in->exponent_den;
  out->approx_order = in->approx_order;
  out->gmp_remez_precision = in->gmp_remez_precision;
  out->error = in->error;
  const double max = minmax[1] * 1.05;
  const double scale = pow(max, power);
  out->RA_a0 = in->RA_a0 * scale;
  for (int k = 0; k < in->approx_order; ++k) {
    out->RA_a[k] = in->RA_a[k] * max * scale;
    out->RA_b[k] = in->RA_b[k] * max;
  }
  out->lambda_min = in->lambda_min * max;
  out->lambda_max = max;
  if (out->lambda_min > minmax[0]) {
    printf("ERROR: mother rational approx does not cover the range!\n");
    printf("out->lambda_max: %e \n", out->lambda_max);
    printf("out->lambda_min: %e , minmax[0]: %e\n", out->lambda_min, minmax[0]);
    printf("Consider modifying your input file, setting\n");
    printf("ExpMaxEigenvalue         %f     # OR LARGER!!\n", max * 1.2);
    printf("Program will now terminate.\n");
    exit(1);
  } else if (out->lambda_min < 0.3 * minmax[0]) {
    printf("Warning, the range of your rational approximation is really large\n");
    printf("out->lambda_min: %e , minmax[0]: %e\n", out->lambda_min, minmax[0]);
    printf("You may consider reducing 'ExpMaxEigenvalue' in the input file to %f.\n", max * 1.2);
  }
}

// The inverse map back to lambda_max = 1 (rationalapprox.c:197-221).
__attribute__((weak)) void renormalize_rational_approximation(RationalApprox* in, RationalApprox* out) {
  const double power = double(in->exponent_num) / in->exponent_den;
  out->exponent_num = in->exponent_num;
  out->exponent_den = in->exponent_den;
  out->approx_order = in->approx_order;
  out->gmp_remez_precision = in->gmp_remez_precision;
  out->error = in->error;
  const double ratio = 1 / in->lambda_max;
  const double scale = pow(ratio, power);
  out->RA_a0 = in->RA_a0 * scale;
  for (int k = 0; k < in->approx_order; ++k) {
    out->RA_a[k] = in->RA_a[k] * ratio * scale;
    out->RA_b[k] = in->RA_b[k] * ratio;
  }
  out->lambda_min = in->lambda_min * ratio;
  out->lambda_max = 1;
}

// r(x) = a0 + sum_i a_i / (x + b_i) (rationalapprox.c:224-236)
__attribute__((weak)) double rational_approx_evaluate(RationalApprox* in, double x) {
  double r = in->RA_a0;
  for (int k = 0; k < in->approx_order; ++k) r += in->RA_a[k] / (x + in->RA_b[k]);
  return r;
}

}  // extern "C"
