// Test driver for marie_gb300/csrc/dense.h (host code): reads a command and
// complex matrices (binary, column-major) from a file, writes the results.
#include <cstdio>
#include <cstring>
#include <vector>

#include "dense.h"

using namespace marie::dense;

static Mat read_mat(FILE* f) {
  int r = 0, c = 0;
  if (std::fread(&r, sizeof(int), 1, f) != 1 || std::fread(&c, sizeof(int), 1, f) != 1) return Mat();
  Mat m(r, c);
  std::vector<double> buf(2 * (size_t)r * c);
  if (std::fread(buf.data(), sizeof(double), buf.size(), f) != buf.size()) return Mat();
  for (size_t i = 0; i < (size_t)r * c; ++i) m.a[i] = cd(buf[2 * i], buf[2 * i + 1]);
  return m;
}
static void write_mat(FILE* f, const Mat& m) {
  std::fwrite(&m.r, sizeof(int), 1, f);
  std::fwrite(&m.c, sizeof(int), 1, f);
  for (const cd& v : m.a) {
    const double re = v.real(), im = v.imag();
    std::fwrite(&re, sizeof(double), 1, f);
    std::fwrite(&im, sizeof(double), 1, f);
  }
}

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  FILE* in = std::fopen(argv[2], "rb");
  FILE* out = std::fopen(argv[3], "wb");
  if (!in || !out) return 3;
  const char* cmd = argv[1];
  if (!std::strcmp(cmd, "eig")) {
    Mat A = read_mat(in), V;
    std::vector<cd> w;
    eig(A, w, V);
    Mat W(A.r, 1);
    for (int i = 0; i < A.r; ++i) W(i, 0) = w[i];
    write_mat(out, W);
    write_mat(out, V);
  } else if (!std::strcmp(cmd, "lstsq")) {
    Mat A = read_mat(in), b = read_mat(in);
    std::vector<cd> x = lstsq(A, b.a);
    Mat X(A.c, 1);
    X.a = x;
    write_mat(out, X);
  } else if (!std::strcmp(cmd, "qr")) {
    Mat A = read_mat(in), Q, R;
    qr_thin(A, Q, R);
    write_mat(out, Q);
    write_mat(out, R);
  } else if (!std::strcmp(cmd, "solve")) {
    Mat A = read_mat(in), B = read_mat(in);
    write_mat(out, solve(A, B));
  } else if (!std::strcmp(cmd, "rdiv")) {
    Mat B = read_mat(in), R = read_mat(in);
    write_mat(out, rdiv_upper(B, R));
  } else {
    return 4;
  }
  std::fclose(in);
  std::fclose(out);
  return 0;
}
