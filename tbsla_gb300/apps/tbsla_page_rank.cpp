// tbsla_page_rank -- the PageRank driver on the GPU library: the flags and
// the report of the reference's driver (src/cpp/apps/tbsla_page_rank.cpp:17-82)
// through the drop-in classes: a Matrix Market file read by
// MatrixCOO::readMM, converted to --format (default COO), then
// Matrix::page_rank (Matrix.cpp:13-61; the GPU sweeps behind it).
//
//   tbsla_page_rank --matrix_input FILE [--beta B (1)] [--epsilon E (1e-5)]
//                   [--max-iterations N (100)] [--format COO|SCOO|CSR|ELL|DENSE]
//                   [--personalized n1,n2,...]
//
// Prints "SOLUTION [b0, b1, b2, b3, ]" and one JSON line with the
// reference's keys (test, matrix_format, n, nnz, nb_iterations, time_read_m,
// time_page_rank, time_app, lang, matrix_input) and the device's name.
#include <algorithm>
#include <cstdlib>
#include <sstream>
#include <vector>

#include <tbsla/cpp/utils/InputParser.hpp>
#include <tbsla/cpp/utils/split.hpp>

#include "driver_common.hpp"

int main(int argc, char **argv) {
  InputParser in(argc, argv);
  const double beta = std::stod(in.get_opt("--beta", "1"));
  const double epsilon = std::stod(in.get_opt("--epsilon", "0.00001"));
  const int max_iterations = std::stoi(in.get_opt("--max-iterations", "100"));
  const std::string format = in.get_opt("--format", "COO");
  const std::string input = in.get_opt("--matrix_input");
  if (input.empty()) {
    std::cerr << "A matrix file has to be given with the parameter --matrix_input file" << std::endl;
    return 1;
  }
  if (!driver::make_matrix(format)) {
    std::cerr << format << " unrecognized!" << std::endl;
    return 1;
  }
  std::vector<int> nodes;
  for (const std::string &t : tbsla::utils::io::split(in.get_opt("--personalized"), ",")) nodes.push_back(std::stoi(t));

  const double t_read0 = driver::seconds();
  tbsla::cpp::MatrixCOO coo;
  coo.readMM(input);
  std::unique_ptr<tbsla::cpp::Matrix> m = driver::convert(coo, format);
  const double t_read1 = driver::seconds();

  int iterations = 0;
  const double t_pr0 = driver::seconds();
  const std::vector<double> b = nodes.empty()
                                    ? m->page_rank(epsilon, beta, max_iterations, iterations)
                                    : m->personalized_page_rank(epsilon, beta, max_iterations, nodes, iterations);
  const double t_pr1 = driver::seconds();

  std::cout << "SOLUTION [";
  for (std::size_t i = 0; i < std::min<std::size_t>(4, b.size()); ++i) std::cout << b[i] << ", ";
  std::cout << "]" << std::endl;

  double peak = 0;
  std::map<std::string, std::string> out;
  out["test"] = nodes.empty() ? "page_rank" : "personalized_page_rank";
  out["matrix_format"] = format;
  out["n"] = std::to_string(m->get_n_col());
  out["nnz"] = std::to_string(m->get_nnz());
  out["nb_iterations"] = std::to_string(iterations);
  out["time_read_m"] = std::to_string(t_read1 - t_read0);
  out["time_page_rank"] = std::to_string(t_pr1 - t_pr0);
  out["time_app"] = std::to_string(driver::seconds() - t_read0);
  out["lang"] = "C++/CUDA";
  out["matrix_input"] = input;
  out["device"] = driver::device_name_and_peak(&peak);
  driver::print_report(out);
  return 0;
}
