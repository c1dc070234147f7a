// post.cpp -- processTLBM.py (python/processTLBM.py) over the dump files, with the unit
// conversion on the GPU (kernels_post.cu), and the XDMF descriptions of its output.
//
// processTLBM stores its datasets in out{n}.h5 / timeAvg.h5 (python/hdf5Helper.py:4-56): the
// same groups and datasets are written here by h5lite.cpp (no HDF5 library), pressure and
// |u| shaped (Nz, Ny, Nx) as processTLBM.py:118-120 reshapes them, the others flat; the XDMF
// files are writeXdmf / writeXdmf_time_avg's (python/hdf5Helper.py:58-202) text.
#include "post.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <fstream>
#include <memory>
#include <sstream>
#include <vector>

#include "engine.h"
#include "h5lite.h"

namespace tlbm {

PostFactors post_factors(const tlbm_problem& p, bool time_avg) {
  PostFactors k;
  const double u_conv = p.t_conv / p.l_conv;  // processTLBM.py:52
  k.u_conv = static_cast<float>(u_conv);
  k.p_conv = static_cast<float>(p.p_conv);
  k.f_conv = static_cast<float>(p.l_conv / (u_conv * u_conv));  // :101
  k.avg = time_avg ? 1 : 0;
  k.avg_div = static_cast<float>(p.num_ts);
  k.p_plane = time_avg ? kPostAvgFields - 1 : kPostPressure;
  return k;
}

int post_num_dumps(const tlbm_problem& p) {
  if (p.plot_freq == 0) return 0;
  const double d = static_cast<double>(p.num_ts - p.warmup_ts) / p.plot_freq;
  return d > 0 ? static_cast<int>(d) : 0;
}

namespace {

std::string fmt(const char* f, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, f);
  std::vsnprintf(buf, sizeof(buf), f, ap);
  va_end(ap);
  return buf;
}

}  // namespace

std::string post_xdmf(const tlbm_problem& p, const std::string& h5_name, bool time_avg) {
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  // x = linspace(0, Lx_p, Nx); dx = x[1] - x[0] = Lx_p / (Nx - 1) (processTLBM.py:54, :62)
  const double dx = nx > 1 ? p.lx_p / (nx - 1) : 0.0;
  auto item = [&](const char* ds) {
    return fmt("<DataItem Dimensions=\"%d %d %d\" NumberType=\"Float\" Format=\"HDF\">\n", nz,
               ny, nx) +
           h5_name + ":/" + ds + "\n</DataItem>\n";
  };
  auto vector = [&](const char* name, const char* const (&ds)[3]) {
    std::string s = fmt("<Attribute Name=\"%s\" AttributeType=\"Vector\" Center=\"Node\">\n", name);
    s += fmt("<DataItem ItemType=\"Function\" Function=\"JOIN($0, $1, $2)\" "
             "Dimensions=\"%d %d %d 3\">\n", nz, ny, nx);
    for (const char* d : ds) s += item(d);
    return s + "</DataItem>\n</Attribute>\n";
  };
  auto scalar = [&](const char* name, const char* ds) {
    return fmt("<Attribute Name=\"%s\" AttributeType=\"Scalar\" Center=\"Node\">\n", name) +
           item(ds) + "</Attribute>\n";
  };
  static const char* const kVelo[3] = {"velo_group/x_velo", "velo_group/y_velo",
                                       "velo_group/z_velo"};
  static const char* const kForce[3] = {"force_group/x_force", "force_group/y_force",
                                        "force_group/z_force"};
  std::string s = "<?xml version=\"1.0\" ?>\n<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" []>\n";
  s += "<Xdmf xmlns:xi=\"http://www.w3.org/2003/XInclude\" Version=\"2.1\">\n<Domain>\n";
  s += "<Grid Name=\"my_Grid\" GridType=\"Uniform\">\n";
  s += fmt("<Topology TopologyType=\"3DCoRectMesh\" Dimensions=\"%d %d %d\">\n</Topology>\n", nz,
           ny, nx);
  s += "<Geometry GeometryType=\"Origin_DxDyDz\">\n";
  s += "<DataItem Dimensions=\"3\" NumberType=\"Integer\" Format=\"XML\">\n0 0 0\n</DataItem>\n";
  s += "<DataItem Dimensions=\"3\" NumberType=\"Integer\" Format=\"XML\">\n";
  s += fmt("%g %g %g\n", dx, dx, dx) + "</DataItem>\n</Geometry>\n";
  s += vector("velocity", kVelo);
  if (!time_avg) s += vector("force", kForce);
  s += scalar("pressure", "pres_group/presmag");
  s += scalar("velocityMagnitude", "velo_group/velmag");
  s += "</Grid>\n</Domain>\n</Xdmf>\n";
  return s;
}

bool post_write(const std::string& dir, const std::string& h5_name, const std::string& xmf_name,
                const tlbm_problem& p, const float* planes, bool time_avg, std::string* err) {
  const uint64_t n = static_cast<uint64_t>(p.nx) * p.ny * p.nz;
  const std::vector<uint64_t> flat = {n};
  const std::vector<uint64_t> grid = {static_cast<uint64_t>(p.nz), static_cast<uint64_t>(p.ny),
                                      static_cast<uint64_t>(p.nx)};
  auto plane = [&](int k) { return planes + static_cast<size_t>(k) * n; };
  std::vector<h5::Dataset> sets = {{"velo_group/x_velo", flat, plane(kPostUx)},
                                   {"velo_group/y_velo", flat, plane(kPostUy)},
                                   {"velo_group/z_velo", flat, plane(kPostUz)},
                                   {"velo_group/velmag", grid, plane(kPostVelmag)}};
  if (!time_avg) {
    sets.push_back({"force_group/x_force", flat, plane(kPostFx)});
    sets.push_back({"force_group/y_force", flat, plane(kPostFy)});
    sets.push_back({"force_group/z_force", flat, plane(kPostFz)});
  }
  sets.push_back({"pres_group/presmag", grid,
                  plane(time_avg ? kPostAvgFields - 1 : kPostPressure)});
  if (!h5::write_f32(dir + "/" + h5_name, sets, err)) return false;
  std::ofstream x(dir + "/" + xmf_name, std::ios::trunc);
  x << post_xdmf(p, h5_name, time_avg);
  if (!x.good()) {
    *err = "write failed: " + dir + "/" + xmf_name;
    return false;
  }
  return true;
}

namespace {

// one raw dump file of n float32 or float64 values
Status read_field(const std::string& path, size_t n, std::vector<char>* buf, int* bytes) {
  std::ifstream in(path, std::ios::binary | std::ios::ate);
  if (!in.is_open()) return Status::err(TLBM_ERR_IO, "cannot open " + path);
  const size_t size = static_cast<size_t>(in.tellg());
  if (size != n * 4 && size != n * 8)
    return Status::err(TLBM_ERR_FORMAT, path + " holds " + std::to_string(size) +
                                            " bytes, not nx*ny*nz float32 or float64 values");
  *bytes = static_cast<int>(size / n);
  buf->resize(size);
  in.seekg(0);
  in.read(buf->data(), static_cast<std::streamsize>(size));
  if (!in.good()) return Status::err(TLBM_ERR_IO, "read failed: " + path);
  return Status::ok();
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

#define POST_CUDA(x)                                                                     \
  do {                                                                                   \
    cudaError_t e_ = (x);                                                                \
    if (e_ != cudaSuccess)                                                               \
      return Status::err(TLBM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

Status post_process_dir(const std::string& dir, int device, int* dumps_done) {
  *dumps_done = 0;
  std::string text;
  Status s = read_text(dir + "/params.lbm", &text);
  if (!s.good()) return s;
  tlbm_problem p{};
  // processTLBM parses every value as a Python float or int (processTLBM.py:27-48)
  s = parse_params(text, false, &p);
  if (!s.good()) return s;
  {
    std::istringstream is(text);
    std::string t;
    int count = 0;
    while (is >> t) ++count;
    if (count < 22)
      return Status::err(TLBM_ERR_FORMAT, "params.lbm: processTLBM needs 22 values (through "
                                          "pRef_idx), found " + std::to_string(count));
  }
  const size_t n = static_cast<size_t>(p.nx) * p.ny * p.nz;
  if (p.p_ref_idx < 0 || static_cast<size_t>(p.p_ref_idx) >= n)
    return Status::err(TLBM_ERR_OUT_OF_RANGE, "params.lbm: pRef_idx outside the lattice");
  std::vector<char> raw;
  int b = 0;
  s = read_field(dir + "/ordering.b_dat", n, &raw, &b);
  if (!s.good()) return s;
  if (b != 4) return Status::err(TLBM_ERR_FORMAT, "ordering.b_dat must hold int32 values");
  const int32_t* order = reinterpret_cast<const int32_t*>(raw.data());
  // the input position that holds node pRef_idx; ordering must be a permutation
  int64_t p_ref_pos = -1;
  {
    std::vector<uint8_t> seen(n, 0);
    for (size_t i = 0; i < n; ++i) {
      const int32_t g = order[i];
      if (g < 0 || static_cast<size_t>(g) >= n || seen[g])
        return Status::err(TLBM_ERR_FORMAT, "ordering.b_dat is not a permutation of the nodes");
      seen[g] = 1;
      if (g == p.p_ref_idx) p_ref_pos = static_cast<int64_t>(i);
    }
  }
  POST_CUDA(cudaSetDevice(device));
  cudaStream_t st = nullptr;
  POST_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  std::unique_ptr<CUstream_st, cudaError_t (*)(cudaStream_t)> st_guard(st, cudaStreamDestroy);
  DevBuf d_order, d_in, d_out;
  POST_CUDA(cudaMalloc(&d_order.p, n * 4));
  POST_CUDA(cudaMemcpy(d_order.p, order, n * 4, cudaMemcpyHostToDevice));
  POST_CUDA(cudaMalloc(&d_in.p, n * 8 * 7));
  POST_CUDA(cudaMalloc(&d_out.p, n * 4 * kPostFields));
  std::vector<float> host(n * kPostFields);
  std::string err;

  auto run = [&](const std::vector<std::string>& names, bool time_avg, const std::string& bin,
                 const std::string& xmf) -> Status {
    int bytes = 0;
    for (size_t k = 0; k < names.size(); ++k) {
      int bk = 0;
      Status r = read_field(dir + "/" + names[k], n, &raw, &bk);
      if (!r.good()) return r;
      if (k > 0 && bk != bytes)
        return Status::err(TLBM_ERR_FORMAT, names[k] + ": element size differs from " + names[0]);
      bytes = bk;
      POST_CUDA(cudaMemcpyAsync(static_cast<char*>(d_in.p) + k * n * bytes, raw.data(),
                                n * bytes, cudaMemcpyHostToDevice, st));
      POST_CUDA(cudaStreamSynchronize(st));  // raw is reused for the next field
    }
    const PostFactors f = post_factors(p, time_avg);
    float* out = static_cast<float*>(d_out.p);
    const int32_t* ord = static_cast<const int32_t*>(d_order.p);
    auto field = [&](auto* base, int k) { return k < (int)names.size() ? base + k * n : nullptr; };
    if (bytes == 4) {
      const float* base = static_cast<const float*>(d_in.p);
      PostInputs<float> in{field(base, 0), field(base, 1), field(base, 2), field(base, 3),
                           field(base, 4), field(base, 5), field(base, 6)};
      POST_CUDA(launch_post(in, ord, static_cast<int64_t>(n), p_ref_pos, f, out, st));
    } else {
      const double* base = static_cast<const double*>(d_in.p);
      PostInputs<double> in{field(base, 0), field(base, 1), field(base, 2), field(base, 3),
                            field(base, 4), field(base, 5), field(base, 6)};
      POST_CUDA(launch_post(in, ord, static_cast<int64_t>(n), p_ref_pos, f, out, st));
    }
    const size_t planes = time_avg ? kPostAvgFields : kPostFields;
    POST_CUDA(cudaMemcpyAsync(host.data(), out, n * 4 * planes, cudaMemcpyDeviceToHost, st));
    POST_CUDA(cudaStreamSynchronize(st));
    if (!post_write(dir, bin, xmf, p, host.data(), time_avg, &err))
      return Status::err(TLBM_ERR_IO, err);
    return Status::ok();
  };

  const int nd = post_num_dumps(p);
  for (int i = 0; i < nd; ++i) {
    const std::string d = std::to_string(i);
    s = run({"ux" + d + ".b_dat", "uy" + d + ".b_dat", "uz" + d + ".b_dat",
             "density" + d + ".b_dat", "Fx" + d + ".b_dat", "Fy" + d + ".b_dat",
             "Fz" + d + ".b_dat"},
            false, "out" + d + ".h5", "data" + d + ".xmf");
    if (!s.good()) return s;
    ++*dumps_done;
  }
  if (p.time_avg_flag == 1) {
    s = run({"uAvg.b_dat", "vAvg.b_dat", "wAvg.b_dat", "rhoAvg.b_dat"}, true, "timeAvg.h5",
            "timeAvg.xmf");
    if (!s.good()) return s;
  }
  return Status::ok();
}

}  // namespace tlbm
