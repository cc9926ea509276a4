// reco_main.cpp -- the reference's MLEM driver flow (reco.cu:32-332) written
// against the drop-in header include/epet_gb300_shim.hpp, single process,
// no MPI.
//
//   epet_reco <measurement> <out> <nrays> <sensitivity> <nIt> <guess|-> <geometry>
//             [--matrix-once | --matrix-free | --csc-transpose]
//
// Files named *.h5 / *.hdf5 are HDF5 as the reference's (read and written by
// the library's own HDF5 code): the measurement is the dataset "messung"
// (readHDF5_MeasVct, wrappers.hpp:311), sensitivity and guess the dataset
// "density" (readHDF5_Density, wrappers.hpp:452), and the output the
// "density" file of writeHDF5_Density (wrappers.hpp:398).  Other names are
// raw float32 files: the measurement dense float[NCHANNELS], the images
// float[V] in voxel-id order.  <geometry> is 20 comma-separated numbers:
// pos0x,pos1x,na,n0z,n0y,n1z,n1y,da,segx,segy,segz, ox,oy,oz,dx,dy,dz,
// nx,ny,nz.  Writes "<it>_<out>" after every iteration as reco.cu does
// (reco.cu:284-291); HDF5 outputs also carry the iterations done (attribute
// "iteration"), and a guess file that carries it resumes the count there:
// iterations it .. nIt-1 run, named as in the uninterrupted run.
//
// Default: the reference's loop -- the system matrix of each row chunk is
// rebuilt in every iteration (reco.cu:216-254).  --matrix-once: the library's
// reconstruction object (matrix built once, iteration in a CUDA graph).
// --matrix-free: the reconstruction object storing no matrix (the chords
// recomputed in every iteration by one walk per row).  --csc-transpose: the
// reference's loop with each chunk's transposed product over its
// column-major copy (epetBuildTranspose) instead of atomics.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/epet_gb300_shim.hpp"

namespace {

// Minimal stand-ins of the reference's geometry value types (same accessors).
struct Grid {
  float o[3], d[3];
  int n[3];
  float gridox() const { return o[0]; }
  float gridoy() const { return o[1]; }
  float gridoz() const { return o[2]; }
  float griddx() const { return d[0]; }
  float griddy() const { return d[1]; }
  float griddz() const { return d[2]; }
  int gridnx() const { return n[0]; }
  int gridny() const { return n[1]; }
  int gridnz() const { return n[2]; }
};
struct Setup {
  float p0, p1, a, sx, sy, sz;
  int na_, n0z_, n0y_, n1z_, n1y_;
  float pos0x() const { return p0; }
  float pos1x() const { return p1; }
  int na() const { return na_; }
  float da() const { return a; }
  int n0z() const { return n0z_; }
  int n0y() const { return n0y_; }
  int n1z() const { return n1z_; }
  int n1y() const { return n1y_; }
  float segx() const { return sx; }
  float segy() const { return sy; }
  float segz() const { return sz; }
};
struct RandRayGen {};  // the per-channel-seeded generator of the library

bool is_h5(const std::string& fn) {
  for (const char* ext : {".h5", ".hdf5"}) {
    const size_t n = strlen(ext);
    if (fn.size() >= n && fn.compare(fn.size() - n, n, ext) == 0) return true;
  }
  return false;
}

// The whole dataset `name` of an HDF5 file, or a raw float32 file; empty if
// the file cannot be read.
std::vector<float> read_f32(const std::string& fn, const char* name) {
  std::vector<float> v;
  if (is_h5(fn)) {
    int32_t nd = 0;
    int64_t dims[8];
    if (epet_h5_dataset_shape(fn.c_str(), name, &nd, dims) != EPET_OK) return v;
    int64_t n = 1;
    for (int i = 0; i < nd; i++) n *= dims[i];
    v.resize(n);
    if (epet_h5_read_f32(fn.c_str(), name, v.data(), n) != EPET_OK) v.clear();
    return v;
  }
  FILE* f = fopen(fn.c_str(), "rb");
  if (!f) return v;
  fseek(f, 0, SEEK_END);
  long n = ftell(f) / 4;
  fseek(f, 0, SEEK_SET);
  v.resize(n);
  if (fread(v.data(), 4, n, f) != (size_t)n) v.clear();
  fclose(f);
  return v;
}

// An image file; HDF5 ones record the iterations done.
bool write_f32(const std::string& fn, const std::vector<float>& v, const epet_grid& g,
               int iterations_done) {
  if (is_h5(fn)) return epet_h5_write_checkpoint(fn.c_str(), v.data(), &g, iterations_done) == EPET_OK;
  FILE* f = fopen(fn.c_str(), "wb");
  if (!f) return false;
  bool ok = fwrite(v.data(), 4, v.size(), f) == v.size();
  fclose(f);
  return ok;
}

#define CK(x) epet_shim::check_cuda((x), #x)

}  // namespace

int main(int argc, char** argv) {
  if (argc < 8) {
    fprintf(stderr,
            "usage: %s measurement out nrays sensitivity nIt guess geometry "
            "[--matrix-once | --matrix-free | --csc-transpose]\n",
            argv[0]);
    return EXIT_FAILURE;
  }
  const std::string fn(argv[1]), on(argv[2]), sfn(argv[4]), xfn(argv[6]);
  const int nrays = atoi(argv[3]), nIt = atoi(argv[5]);
  const std::string mode = argc > 8 ? std::string(argv[8]) : std::string();
  const bool once = mode == "--matrix-once", free_ = mode == "--matrix-free";
  const bool csc_t = mode == "--csc-transpose";
  double g[20];
  {
    std::stringstream ss(argv[7]);
    std::string tok;
    for (int i = 0; i < 20; i++) {
      if (!std::getline(ss, tok, ',')) {
        fprintf(stderr, "geometry needs 20 numbers\n");
        return EXIT_FAILURE;
      }
      g[i] = atof(tok.c_str());
    }
  }
  Setup setup{(float)g[0], (float)g[1], (float)g[7], (float)g[8], (float)g[9], (float)g[10],
              (int)g[2], (int)g[3], (int)g[4], (int)g[5], (int)g[6]};
  Grid grid{{(float)g[11], (float)g[12], (float)g[13]},
            {(float)g[14], (float)g[15], (float)g[16]},
            {(int)g[17], (int)g[18], (int)g[19]}};
  const int V = grid.n[0] * grid.n[1] * grid.n[2];
  const epet_grid egrid{{grid.o[0], grid.o[1], grid.o[2]},
                        {grid.d[0], grid.d[1], grid.d[2]},
                        {grid.n[0], grid.n[1], grid.n[2]}};
  const long NCH = (long)setup.na_ * setup.n0z_ * setup.n0y_ * setup.n1z_ * setup.n1y_;
  try {
    epetSetConstantGeometry(grid, setup, nrays);

    // measurement -> (row ids ascending, values), zero channels dropped
    std::vector<float> meas = read_f32(fn, "messung");
    if ((long)meas.size() != NCH) {
      fprintf(stderr, "measurement must hold %ld floats\n", NCH);
      return EXIT_FAILURE;
    }
    std::vector<int> yRowId;
    std::vector<float> yVal;
    for (long i = 0; i < NCH; i++)
      if (meas[i] != 0.f) {
        yRowId.push_back((int)i);
        yVal.push_back(meas[i]);
      }
    const int effM = (int)yRowId.size();
    int* yRowId_devi = nullptr;
    float* yVal_devi = nullptr;
    CK(cudaMalloc((void**)&yRowId_devi, sizeof(int) * std::max(effM, 1)));
    CK(cudaMalloc((void**)&yVal_devi, sizeof(float) * std::max(effM, 1)));
    CK(cudaMemcpy(yRowId_devi, yRowId.data(), sizeof(int) * effM, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(yVal_devi, yVal.data(), sizeof(float) * effM, cudaMemcpyHostToDevice));

    // density guess or homogeneous, normalised (reco.cu:113-137)
    std::vector<float> x_host = read_f32(xfn, "density");
    const bool xgood = (int)x_host.size() == V;
    int it0 = 0;  // iterations already done (a checkpoint guess)
    if (xgood && is_h5(xfn)) {
      double v = 0.0;
      if (epet_h5_read_attribute(xfn.c_str(), "density", "iteration", &v) == EPET_OK && v > 0)
        it0 = (int)v;
    }
    if (!xgood) x_host.assign(V, 1.f);
    float* x_devi = nullptr;
    CK(cudaMalloc((void**)&x_devi, sizeof(float) * V));
    CK(cudaMemcpy(x_devi, x_host.data(), sizeof(float) * V, cudaMemcpyHostToDevice));
    if (!xgood) {
      float norm = sum<float>(x_devi, V);
      scales<float>(x_devi, (float)(1. / norm), V);
    }
    // sensitivity, normalised (reco.cu:150-183)
    std::vector<float> s_host = read_f32(sfn, "density");
    if ((int)s_host.size() != V) {
      fprintf(stderr, "sensitivity must hold %d floats\n", V);
      return EXIT_FAILURE;
    }
    float* s_devi = nullptr;
    CK(cudaMalloc((void**)&s_devi, sizeof(float) * V));
    CK(cudaMemcpy(s_devi, s_host.data(), sizeof(float) * V, cudaMemcpyHostToDevice));
    {
      float norm = sum<float>(s_devi, V);
      scales<float>(s_devi, (float)(1. / norm), V);
    }

    if (once || free_) {
      epet_problem p;
      epet_shim::check(epet_get_constant_geometry(&p), "geometry");
      epet_mlem_options o{0, 1, 0, 0, free_ ? 1 : 0};
      epet_mlem* h = nullptr;
      epet_shim::check(epet_mlem_create(&p, yRowId_devi, yVal_devi, effM, s_devi, &o, &h, 0),
                       "epet_mlem_create");
      if (xgood) epet_shim::check(epet_mlem_set_image(h, x_devi, 0), "set image");
      for (int it = it0; it < nIt; it++) {
        double ll = 0;
        epet_shim::check(epet_mlem_iterate(h, 1, &ll, 0), "iterate");
        epet_shim::check(epet_mlem_get_image(h, x_devi, 0), "image");
        CK(cudaMemcpy(x_host.data(), x_devi, sizeof(float) * V, cudaMemcpyDeviceToHost));
        std::stringstream ss;
        ss << it;
        write_f32(ss.str() + "_" + on, x_host, egrid, it + 1);
        printf("it %d loglik %.9g\n", it, ll);
      }
      epet_mlem_destroy(h);
      return 0;
    }

    // the reference's loop: chunks of LIMM rows, matrix rebuilt per chunk and
    // iteration (reco.cu:24-30, :209-254)
    const unsigned long long LIMNNZ = (512ull * 1024 * 1024) / sizeof(float);
    const int LIMM = (int)(LIMNNZ / V);
    float *yt = nullptr, *e = nullptr, *c = nullptr, *xx = nullptr, *val = nullptr;
    int *cnl = nullptr, *csr = nullptr, *ecsr = nullptr, *vxl = nullptr;
    unsigned long long* nnz_devi = nullptr;
    CK(cudaMalloc((void**)&yt, sizeof(float) * LIMM));
    CK(cudaMalloc((void**)&e, sizeof(float) * LIMM));
    CK(cudaMalloc((void**)&c, sizeof(float) * V));
    CK(cudaMalloc((void**)&xx, sizeof(float) * V));
    CK(cudaMalloc((void**)&cnl, sizeof(int) * (size_t)LIMM * V));
    CK(cudaMalloc((void**)&csr, sizeof(int) * (NCH + 1)));
    CK(cudaMalloc((void**)&ecsr, sizeof(int) * (LIMM + 1)));
    CK(cudaMalloc((void**)&vxl, sizeof(int) * (size_t)LIMM * V));
    CK(cudaMalloc((void**)&val, sizeof(float) * (size_t)LIMM * V));
    CK(cudaMalloc((void**)&nnz_devi, sizeof(unsigned long long)));
    cusparseHandle_t handle = nullptr;
    cusparseMatDescr_t A = nullptr;
    float zero = 0.f, one = 1.f;
    const unsigned NChunks =
        nChunks<unsigned, unsigned long long>((unsigned long long)effM * V,
                                              (unsigned long long)LIMM * V);
    for (int it = it0; it < nIt; it++) {
      CK(cudaMemset(c, 0, sizeof(float) * V));
      for (unsigned chunkId = 0; chunkId < NChunks; chunkId++) {
        unsigned m = nInChunk<unsigned, unsigned>(chunkId, effM, LIMM);
        unsigned ptr = chunkPtr<unsigned, unsigned>(chunkId, LIMM);
        unsigned long long nnz_host = 0;
        CK(cudaMemcpy(nnz_devi, &nnz_host, sizeof(nnz_host), cudaMemcpyHostToDevice));
        const unsigned* mp = &m;
        systemMatrixCalculation<float, unsigned, int, unsigned long long, RandRayGen>(
            ecsr, vxl, val, nnz_devi, cnl, csr, &yRowId_devi[ptr], mp, handle);
        CK(cudaMemcpy(&nnz_host, nnz_devi, sizeof(nnz_host), cudaMemcpyDeviceToHost));
        CSRmv<float>()(handle, CUSPARSE_OPERATION_NON_TRANSPOSE, m, V, (int)nnz_host, &one, A,
                       val, ecsr, vxl, x_devi, &zero, yt);
        float* yv = &yVal_devi[ptr];
        divides<float>(e, yv, yt, m);
        // --csc-transpose: the chunk's column-major copy makes the transposed
        // product scatter-free (deterministic) instead of atomic
        if (csc_t) epetBuildTranspose(m, V, (int)nnz_host, val, ecsr, vxl);
        CSRmv<float>()(handle, CUSPARSE_OPERATION_TRANSPOSE, m, V, (int)nnz_host, &one, A, val,
                       ecsr, vxl, e, &one, c);
        if (csc_t) epetReleaseTranspose(val);
      }
      dividesMultiplies<float>(xx, x_devi, c, s_devi, V);
      CK(cudaMemcpy(x_devi, xx, sizeof(float) * V, cudaMemcpyDeviceToDevice));
      float norm = sum<float>(x_devi, V);
      scales<float>(x_devi, (float)(1. / norm), V);
      CK(cudaMemcpy(x_host.data(), x_devi, sizeof(float) * V, cudaMemcpyDeviceToHost));
      std::stringstream ss;
      ss << it;
      write_f32(ss.str() + "_" + on, x_host, egrid, it + 1);
      printf("it %d norm %.9g\n", it, (double)sum<float>(x_devi, V));
    }
    return 0;
  } catch (cudaException&) {
    return EXIT_FAILURE;
  }
}
