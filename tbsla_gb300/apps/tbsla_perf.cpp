// tbsla_perf -- the SpMV benchmark driver on the GPU library: the flags and
// report of the reference's driver (src/cpp/apps/tbsla_perf.cpp:27-194)
// through the drop-in classes, plus the GPU's own figures.
//
//   tbsla_perf --format COO|SCOO|CSR|ELL|DENSE --matrix cdiag|cqmat|NAME
//              [--NR 1024] [--NC 1024] [--C 8] [--Q 0.1] [--S 0]
//              [--matrix_folder .] --op spmv|spmv_no_redist|Ax|Ax_|a_axpx
//              [--print-infos] [--reps 10]
//
// The matrix is filled by the reference's generators (fill_cdiag /
// fill_cqmat, whole matrix) or read from MATRIX_FOLDER/NAME.FORMAT
// (Matrix::read), and multiplied by x uniform in [-1, 1) (seeded).  Keys as
// the reference's (test, matrix_format, n_row, n_col, nnz, time_app_in,
// time_op, gflops, lang, matrix_type, compiler, compile_options, cdiag_c /
// cqmat_c / cqmat_q / cqmat_s), time_op being the drop-in call with host
// vectors (x copied in, the result copied out), as the reference's call is
// timed.  Added: time_op_device (the same operation on vectors resident in
// device memory, the mean of --reps calls), gbps and gbps_device
// (algorithmic bytes: stored entries with their indices, the row pointer,
// x read and y written once; a_axpx twice the matrix and five vectors),
// peak_gbs (the device's theoretical HBM rate), roofline_frac
// (gbps_device / peak_gbs) and device.
#include <random>
#include <vector>

#include <tbsla/Configs.h>
#include <tbsla/cpp/utils/InputParser.hpp>

#include "driver_common.hpp"

int main(int argc, char **argv) {
  InputParser in(argc, argv);
  const std::string format = in.get_opt("--format");
  if (format.empty()) {
    std::cerr << "A file format has to be given with the parameter --format format" << std::endl;
    return 1;
  }
  const int NR = std::stoi(in.get_opt("--NR", "1024")), NC = std::stoi(in.get_opt("--NC", "1024"));
  const std::string matrix = in.get_opt("--matrix"), folder = in.get_opt("--matrix_folder", ".");
  int C = -1, S = -1;
  double Q = -1;
  if (matrix == "cdiag") {
    C = std::stoi(in.get_opt("--C", "8"));
  } else if (matrix == "cqmat") {
    C = std::stoi(in.get_opt("--C", "8"));
    Q = std::stod(in.get_opt("--Q", "0.1"));
    S = std::stoi(in.get_opt("--S", "0"));
  } else if (matrix.empty()) {
    std::cerr << "No matrix has been given with the parameter --matrix matrix." << std::endl;
    return 1;
  }
  const std::string op = in.get_opt("--op");
  if (op.empty()) {
    std::cerr << "An operation (spmv, a_axpx) has to be given with the parameter --op op" << std::endl;
    return 1;
  }
  if (op != "spmv" && op != "a_axpx" && op != "spmv_no_redist" && op != "Ax" && op != "Ax_") {
    std::cerr << "OP : " << op << " unrecognized!" << std::endl;
    return 1;
  }
  const int reps = std::max(1, std::stoi(in.get_opt("--reps", "10")));
  std::unique_ptr<tbsla::cpp::Matrix> m = driver::make_matrix(format);
  if (!m) {
    std::cerr << format << " unrecognized!" << std::endl;
    return 1;
  }
  const double t_app0 = driver::seconds();
  if (matrix == "cdiag") {
    m->fill_cdiag(NR, NC, C, 0, 0, 1, 1);
  } else if (matrix == "cqmat") {
    m->fill_cqmat(NR, NC, C, Q, S, 0, 0, 1, 1);
  } else {
    std::ifstream is(folder + "/" + matrix + "." + format, std::ifstream::binary);
    m->read(is);
  }
  if (in.has_opt("--print-infos")) {
    m->print_stats(std::cout);
    m->print_infos(std::cout);
  }
  std::mt19937 gen(12345);
  std::uniform_real_distribution<double> dist(-1, 1);
  std::vector<double> x((size_t)m->get_n_col()), r((size_t)m->get_n_row(), 0.0);
  for (double &v : x) v = dist(gen);
  const bool axpx = op == "a_axpx";

  // the drop-in call with host vectors (the device copy is built first, as
  // the reference's matrix is already in memory when its call is timed)
  tbsla_matrix_t *h = m->device_matrix();
  const double t_op0 = driver::seconds();
  if (op == "spmv" || op == "spmv_no_redist") {
    std::vector<double> y = m->spmv(x);
  } else if (op == "Ax" || op == "Ax_") {
    m->Ax(r, x);
  } else {
    std::vector<double> y = m->a_axpx_(x);
  }
  const double t_op1 = driver::seconds();
  const double t_app1 = driver::seconds();

  // the same operation on device-resident vectors
  double t_dev = 0;
  tbsla_matrix_info_t info{};
  const bool have_device = h && tbsla_matrix_info(h, &info) == TBSLA_OK;
  if (have_device) {
    const int64_t nx = std::max<int64_t>(m->get_n_col(), 1), ny = std::max<int64_t>(m->get_n_row(), 1);
    void *dx = nullptr, *dy = nullptr, *dt = nullptr;
    tbsla_device_alloc(&dx, (size_t)std::max(nx, ny) * 8);
    tbsla_device_alloc(&dy, (size_t)std::max(nx, ny) * 8);
    tbsla_device_alloc(&dt, (size_t)std::max(nx, ny) * 8);
    tbsla_memcpy_h2d(dx, x.data(), (size_t)nx * 8, nullptr);
    auto run = [&] {
      return axpx ? tbsla_a_axpx(h, (const double *)dx, (double *)dy, (double *)dt, 0, nullptr)
                  : tbsla_spmv(h, (const double *)dx, (double *)dy, 0, nullptr);
    };
    tbsla_status_t st = run();
    tbsla_stream_sync(nullptr);
    const double d0 = driver::seconds();
    for (int k = 0; k < reps && st == TBSLA_OK; ++k) st = run();
    tbsla_stream_sync(nullptr);
    t_dev = st == TBSLA_OK ? (driver::seconds() - d0) / reps : 0;
    tbsla_device_free(dx);
    tbsla_device_free(dy);
    tbsla_device_free(dt);
  }

  double peak = 0;
  const std::string device = driver::device_name_and_peak(&peak);
  double bytes = have_device ? driver::product_bytes(info) : 0;
  if (axpx) bytes = 2 * (bytes - 8.0 * ((double)info.n_col + info.n_row)) + 5 * 8.0 * (double)info.n_row;
  std::map<std::string, std::string> out;
  out["test"] = op;
  out["matrix_format"] = format;
  out["n_row"] = std::to_string(m->get_n_row());
  out["n_col"] = std::to_string(m->get_n_col());
  out["nnz"] = std::to_string(m->get_nnz());
  out["time_app_in"] = std::to_string(t_app1 - t_app0);
  out["time_op"] = std::to_string(t_op1 - t_op0);
  out["gflops"] = std::to_string((axpx ? 4.0 : 2.0) * m->get_nnz() / ((t_op1 - t_op0) * 1e9));
  out["lang"] = "C++/CUDA";
  out["matrix_type"] = matrix;
  out["compiler"] = std::string(CMAKE_CXX_COMPILER_ID) + " " + std::string(CMAKE_CXX_COMPILER_VERSION);
  out["compile_options"] = std::string(CMAKE_BUILD_TYPE) + " " + std::string(CMAKE_CXX_FLAGS_RELEASE);
  if (matrix == "cdiag") {
    out["cdiag_c"] = std::to_string(C);
  } else if (matrix == "cqmat") {
    out["cqmat_c"] = std::to_string(C);
    out["cqmat_q"] = std::to_string(Q);
    out["cqmat_s"] = std::to_string(S);
  }
  out["device"] = device;
  out["time_op_device"] = std::to_string(t_dev);
  out["gbps"] = std::to_string(bytes / (t_op1 - t_op0) / 1e9);
  out["gbps_device"] = std::to_string(t_dev > 0 ? bytes / t_dev / 1e9 : 0.0);
  out["peak_gbs"] = std::to_string(peak);
  out["roofline_frac"] = std::to_string(t_dev > 0 && peak > 0 ? bytes / t_dev / 1e9 / peak : 0.0);
  driver::print_report(out);
  return 0;
}
