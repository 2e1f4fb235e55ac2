// Density files of the reference (host code, no GPU needed):
//   cdft_density_write / cdft_density_read  Density::writeDensity / readDensity
//     (src/Density.cpp:227-244): the real density vector saved by Armadillo's
//     Col<double>::save in its default arma_binary format, i.e. the text header
//     line "ARMA_MAT_BIN_FN008", a line "<n_rows> <n_cols>" (n 1 for a column
//     vector), then the n values as raw native doubles (Armadillo's published
//     format; the reference links Armadillo for its DFT_Vec storage,
//     additionalCode/DFT_Armadillo.cpp:86-87).
//   cdft_density_write_vtk  Density::write_VTK_File (src/Density.cpp:197-225):
//     the reference's VisIt writer (src/visit_writer.cpp, write_regular_mesh
//     with useBinary = 0) produces a legacy-VTK ASCII rectilinear grid with
//     (Nx+1)(Ny+1)(Nz+1) points at integer coordinates and the density as one
//     cell-centred float scalar, x fastest; floats are printed "%20.12e " nine
//     to a line. The same bytes are produced here (checked against files the
//     reference itself wrote).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cdft.h"

namespace {

const char kArmaHeader[] = "ARMA_MAT_BIN_FN008";

// Prints floats as the VisIt writer does: "%20.12e " each, a newline after
// every ninth, and a newline to close a section that ended mid-line.
struct FloatLines {
  FILE* f;
  int col = 0;
  void put(float v) {
    std::fprintf(f, "%20.12e ", (double)v);
    if (++col == 9) {
      std::fputc('\n', f);
      col = 0;
    }
  }
  void close_section() {  // only when the last line is open
    if (col != 0) std::fputc('\n', f);
    col = 0;
  }
  void end_block() {  // unconditional newline after a variable's values
    std::fputc('\n', f);
    col = 0;
  }
};

}  // namespace

extern "C" {

int cdft_density_write(const char* path, const double* rho, long n) {
  if (!path || !rho || n <= 0) return CDFT_ERR_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return CDFT_ERR_ARG;
  std::fprintf(f, "%s\n%ld 1\n", kArmaHeader, n);
  const size_t w = std::fwrite(rho, sizeof(double), (size_t)n, f);
  const int bad = std::fclose(f);
  return (w == (size_t)n && bad == 0) ? CDFT_OK : CDFT_ERR_ARG;
}

int cdft_density_read(const char* path, double* rho, long n) {
  if (!path || !rho || n <= 0) return CDFT_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return CDFT_ERR_ARG;  // the reference throws "Could not open input file"
  char head[64] = {0};
  long rows = -1, cols = -1;
  int ok = std::fscanf(f, "%63s", head) == 1 && std::strcmp(head, kArmaHeader) == 0 &&
           std::fscanf(f, "%ld %ld", &rows, &cols) == 2 && std::fgetc(f) == '\n';
  ok = ok && rows * cols == n && (rows == 1 || cols == 1);
  if (ok) ok = std::fread(rho, sizeof(double), (size_t)n, f) == (size_t)n;
  std::fclose(f);
  return ok ? CDFT_OK : CDFT_ERR_ARG;
}

int cdft_density_write_vtk(const char* path, const double* rho, int nx, int ny, int nz) {
  if (!path || !rho || nx <= 0 || ny <= 0 || nz <= 0) return CDFT_ERR_ARG;
  std::string name(path);
  if (name.find(".vtk") == std::string::npos) name += ".vtk";
  FILE* f = std::fopen(name.c_str(), "w");
  if (!f) return CDFT_ERR_ARG;
  const int dims[3] = {nx + 1, ny + 1, nz + 1};
  const long ncells = (long)nx * ny * nz, npts = (long)dims[0] * dims[1] * dims[2];
  std::fprintf(f, "# vtk DataFile Version 2.0\nWritten using VisIt writer\nASCII\n");
  std::fprintf(f, "DATASET RECTILINEAR_GRID\nDIMENSIONS %d %d %d\n", dims[0], dims[1], dims[2]);
  FloatLines out{f};
  const char axis[3] = {'X', 'Y', 'Z'};
  for (int a = 0; a < 3; ++a) {
    if (a > 0) out.close_section();
    std::fprintf(f, "%c_COORDINATES %d float\n", axis[a], dims[a]);
    for (int i = 0; i < dims[a]; ++i) out.put((float)i);
  }
  out.close_section();
  std::fprintf(f, "CELL_DATA %ld\nSCALARS density float\nLOOKUP_TABLE default\n", ncells);
  for (int k = 0; k < nz; ++k)  // x fastest, as the reference fills its float buffer
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) out.put((float)rho[k + (long)nz * (j + (long)ny * i)]);
  out.end_block();
  std::fprintf(f, "POINT_DATA %ld\n", npts);
  std::fputc('\n', f);  // the writer ends an ASCII file with one more newline
  return std::fclose(f) == 0 ? CDFT_OK : CDFT_ERR_ARG;
}

}  // extern "C"
