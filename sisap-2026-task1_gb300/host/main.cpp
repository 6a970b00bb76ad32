// main.cpp -- knng_main: drop-in CLI for the reference engine's process
// interface (Aftab5550/SISAP-2026-task1 src/main.cpp:114-498).
//
//   knng_main --task task1 --dataset data/X.h5 [options]
//
// Same argv rules (src/main.cpp:124-133: --dataset F, --task T defaulting to
// task1, else the first bare argument is the dataset), same progress lines,
// same result file results/<task>/apex_simd.h5 with knns/dists and the
// attributes algo, task, buildtime, querytime, params (:459-480), same -1 exit
// status on failure (:140, 197, 200, 484, 487).  The graph is built on the GPU
// through the libknng C ABI.  Extra options (all default to the reference's
// compile-time constants, src/main.cpp:19-29):
//   --k-build K --k-eval k --trees T --leaf L --rerank M --max-iter I
//   --quant trunc|round --join jacobi|inplace --order leaf|natural
//   --device D --stats-json FILE
//   --output-format hdf5|knng   (result file format; hdf5 by default)
// and an inspection mode that needs no GPU:
//   knng_main --h5dump FILE [DATASET]   prints the file's datasets and root
//   attributes (and DATASET's values as float32) as one JSON object;
//   knng_main --convert SRC DST [--output-format hdf5|knng]   rewrites a
//   result file (knns, dists, attributes) in the other format;
//   knng_main --pca SRC DST DIMS [--device D]   PCA preprocessing on the GPU
//   (scripts/data_prep/apply_pca.py): /train projected to DIMS components,
//   L2-normalised, written as float16, with /allknn/knns and /allknn/dists
//   copied from an HDF5 SRC when present.
#include <sys/stat.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "h5io.h"
#include "hdf5.h"
#include "knng.h"

namespace {

std::string json_str(const std::string& s) {
  std::string o = "\"";
  for (unsigned char ch : s) {
    if (ch == '"' || ch == '\\') {
      o += '\\';
      o += char(ch);
    } else if (ch < 0x20) {
      char b[8];
      std::snprintf(b, sizeof b, "\\u%04x", ch);
      o += b;
    } else {
      o += char(ch);
    }
  }
  return o + "\"";
}

int h5dump(const std::string& path, const std::string& dataset) {
  try {
    std::string out = "{\"datasets\": [";
    const auto ds = knngio::h5::list_datasets(path);
    for (size_t i = 0; i < ds.size(); ++i) {
      out += (i ? ", " : "") + std::string("{\"name\": ") + json_str(ds[i].name) +
             ", \"class\": " + std::to_string(ds[i].type_class) + ", \"size\": " + std::to_string(ds[i].type_size) +
             ", \"little_endian\": " + (ds[i].little_endian ? "true" : "false") +
             ", \"signed\": " + (ds[i].is_signed ? "true" : "false") + ", \"dims\": [";
      for (size_t k = 0; k < ds[i].dims.size(); ++k) out += (k ? ", " : "") + std::to_string(ds[i].dims[k]);
      out += "]}";
    }
    out += "], \"attrs\": {";
    const auto at = knngio::h5::read_attributes(path, "/");
    for (size_t i = 0; i < at.size(); ++i) out += (i ? ", " : "") + json_str(at[i].first) + ": " + json_str(at[i].second);
    out += "}";
    if (!dataset.empty()) {
      const std::vector<float> v = knngio::h5::read_float(path, dataset, nullptr);
      out += ", \"values\": [";
      char b[32];
      for (size_t i = 0; i < v.size(); ++i) {
        std::snprintf(b, sizeof b, "%s%.9g", i ? ", " : "", double(v[i]));
        out += b;
      }
      out += "]";
    }
    std::cout << out << "}\n";
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "[FATAL] " << e.what() << "\n";
    return -1;
  }
}

bool take_int(const std::string& a, const char* flag, int argc, char** argv, int& i, int& out) {
  if (a != flag || i + 1 >= argc) return false;
  out = std::atoi(argv[++i]);
  return true;
}

std::string fmt_params(const knng_params& p) {
  std::ostringstream s;
  s << "K_BUILD=" << p.k_build << ", RERANK=" << p.rerank_mult << ", TREES=" << p.num_trees
    << ", LEAF=" << p.leaf_size << ", STOP=" << p.early_stop_rate << ", DIFF=" << p.rate_diff_tol;
  return s.str();
}

}  // namespace

int convert(const std::string& src, const std::string& dst, knngio::Format format) {
  try {
    const knngio::Result r = knngio::read_result(src);
    const knngio::Output o{r.knns.data(), r.dists.data(), r.rows, r.cols, r.algo, r.task, r.params, r.buildtime,
                           r.querytime};
    knngio::write_result(dst, o, format);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "[FATAL] " << e.what() << "\n";
    return -1;
  }
}

int pca(const std::string& src, const std::string& dst, int dims, int device) {
  try {
    const auto t0 = std::chrono::steady_clock::now();
    const knngio::Matrix m = knngio::read_matrix(src, "/train");
    std::cout << "[1] Loaded /train: " << m.rows << " x " << m.cols << "\n";
    std::vector<uint16_t> out(size_t(m.rows) * size_t(dims));
    double kept = 0.0;
    const int st = knng_pca(m.data.data(), m.rows, int(m.cols), dims, device, out.data(), &kept);
    if (st != KNNG_OK) {
      std::cerr << "[FATAL] PCA: " << knng_status_string(st) << "\n";
      return -1;
    }
    std::cout << "  -> Variance Retained: " << kept * 100.0 << "%\n";
    std::vector<knngio::h5::WriteDataset> ds = {{"train", 2, {uint64_t(m.rows), uint64_t(dims)}, out.data()}};
    std::vector<int32_t> gk;
    std::vector<float> gd;
    knngio::h5::DatasetInfo ki, di;
    if (knngio::h5::is_hdf5(src)) {
      for (const auto& d : knngio::h5::list_datasets(src)) {
        if (d.name == "allknn/knns") gk = knngio::h5::read_int32(src, d.name, &ki);
        if (d.name == "allknn/dists") gd = knngio::h5::read_float(src, d.name, &di);
      }
    }
    if (!gk.empty()) ds.push_back({"allknn/knns", 0, ki.dims, gk.data()});
    if (!gd.empty()) ds.push_back({"allknn/dists", 1, di.dims, gd.data()});
    knngio::h5::write_file(dst, ds, {});
    const std::chrono::duration<double> dt = std::chrono::steady_clock::now() - t0;
    std::cout << "  -> Saved " << dst << (gk.empty() ? "" : " (with /allknn)") << " in " << dt.count() << " s\n";
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "[FATAL] " << e.what() << "\n";
    return -1;
  }
}

int main(int argc, char** argv) {
  if (argc >= 3 && std::string(argv[1]) == "--h5dump") return h5dump(argv[2], argc >= 4 ? argv[3] : "");
  if (argc >= 5 && std::string(argv[1]) == "--pca") {
    const int device = (argc >= 7 && std::string(argv[5]) == "--device") ? std::atoi(argv[6]) : 0;
    return pca(argv[2], argv[3], std::atoi(argv[4]), device);
  }
  if (argc >= 4 && std::string(argv[1]) == "--convert") {
    const bool knng = argc >= 6 && std::string(argv[4]) == "--output-format" && std::string(argv[5]) == "knng";
    return convert(argv[2], argv[3], knng ? knngio::Format::kContainer : knngio::Format::kHdf5);
  }
  const auto global_start = std::chrono::steady_clock::now();
  std::cout << "==================================================\n";
  std::cout << "   KNNG GB300 ENGINE: kNN-GRAPH BUILD ON ONE GPU   \n";
  std::cout << "==================================================\n";

  std::string filename, task_name = "task1", stats_json;
  knngio::Format out_format = knngio::Format::kHdf5;
  knng_params prm;
  knng_default_params(&prm);
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (take_int(a, "--k-build", argc, argv, i, prm.k_build) || take_int(a, "--k-eval", argc, argv, i, prm.k_eval) ||
        take_int(a, "--trees", argc, argv, i, prm.num_trees) || take_int(a, "--leaf", argc, argv, i, prm.leaf_size) ||
        take_int(a, "--rerank", argc, argv, i, prm.rerank_mult) ||
        take_int(a, "--max-iter", argc, argv, i, prm.max_iterations) ||
        take_int(a, "--device", argc, argv, i, prm.device)) {
      continue;
    }
    if (a == "--quant" && i + 1 < argc) {
      prm.quant_mode = std::string(argv[++i]) == "round" ? KNNG_QUANT_ROUND : KNNG_QUANT_TRUNC;
    } else if (a == "--join" && i + 1 < argc) {
      prm.join_mode = std::string(argv[++i]) == "inplace" ? KNNG_JOIN_INPLACE : KNNG_JOIN_JACOBI;
    } else if (a == "--order" && i + 1 < argc) {
      prm.row_order = std::string(argv[++i]) == "natural" ? KNNG_ORDER_NATURAL : KNNG_ORDER_LEAF;
    } else if (a == "--output-format" && i + 1 < argc) {
      out_format = std::string(argv[++i]) == "knng" ? knngio::Format::kContainer : knngio::Format::kHdf5;
    } else if (a == "--stats-json" && i + 1 < argc) {
      stats_json = argv[++i];
    } else if (a == "--dataset" && i + 1 < argc) {
      filename = argv[++i];
    } else if (a == "--task" && i + 1 < argc) {
      task_name = argv[++i];
    } else if (filename.empty() && a.find("--") != 0) {
      filename = a;
    }
  }
  std::cout << "[INFO] Target Dataset: " << filename << "\n";
  std::cout << "[INFO] Target Task: " << task_name << "\n";
  if (filename.empty()) {
    std::cerr << "[FATAL] No filename provided.\n";
    return -1;
  }

  knngio::Matrix train;
  std::cout << "[INFO] Inspecting dataset metadata...\n";
  try {
    train = knngio::read_matrix(filename, "/train");
  } catch (const std::exception& e) {
    std::cerr << "[FATAL] Dataset Error: " << e.what() << "\n";
    return -1;
  }
  std::cout << "[OK] Detected " << train.rows << " vectors in /train.\n";

  knng_ctx* ctx = nullptr;
  int st = knng_create(&ctx, &prm);
  if (st != KNNG_OK) {
    std::cerr << "[FATAL] GPU context: " << knng_status_string(st) << "\n";
    return -1;
  }
  const int64_t n = train.rows;
  std::vector<int32_t> knns(size_t(n) * prm.k_eval);
  std::vector<float> dists(size_t(n) * prm.k_eval);
  knng_stats stats{};
  std::cout << "[INFO] Building kNN graph on the GPU (quantise, RP forest, leaf init, NN-Descent)...\n";
  st = knng_build(ctx, train.data.data(), n, int(train.cols), 0, knns.data(), dists.data(), 0, &stats);
  if (st != KNNG_OK) {
    std::cerr << "[FATAL] Build Error: " << knng_status_string(st) << ": " << knng_last_error(ctx) << "\n";
    knng_destroy(ctx);
    return -1;
  }
  knng_destroy(ctx);
  std::cout << "[OK] Forest constructed (" << stats.forest_levels << " levels, " << stats.leaves << " leaves).\n";
  std::cout << "[OK] Graph Initialization Complete.\n";
  for (int it = 0; it < stats.iterations && it < 64; ++it) {
    const float rate = float(stats.updates[it]) / float(uint64_t(n) * uint64_t(prm.k_build));
    std::cout << "  -> Iteration " << it + 1 << " Updates: " << stats.updates[it] << " (Rate: " << rate * 100.0f
              << "%)\n";
  }
  std::cout << "[INFO] Exporting Results...\n";

  mkdir("results", 0777);
  const std::string res_dir = "results/" + task_name;
  mkdir(res_dir.c_str(), 0777);
  const std::string out_filename = res_dir + "/apex_simd.h5";
  try {
    knngio::Output o{knns.data(), dists.data(), n, prm.k_eval, "knng GB300", task_name, fmt_params(prm),
                     float(stats.build_s), 0.0f};
    knngio::write_result(out_filename, o, out_format);
  } catch (const std::exception& e) {
    std::cerr << "[FATAL] File Write Error: " << e.what() << "\n";
    return -1;
  }
  if (!stats_json.empty()) {
    if (FILE* f = std::fopen(stats_json.c_str(), "w")) {
      std::fprintf(f,
                   "{\"n\": %lld, \"d\": %lld, \"quantize_s\": %.6f, \"forest_s\": %.6f, \"init_s\": %.6f, "
                   "\"join_s\": %.6f, \"export_s\": %.6f, \"build_s\": %.6f, \"total_s\": %.6f, \"iterations\": %d}\n",
                   (long long)n, (long long)train.cols, stats.quantize_s, stats.forest_s, stats.init_s, stats.join_s,
                   stats.export_s, stats.build_s, stats.total_s, stats.iterations);
      std::fclose(f);
    }
  }
  const std::chrono::duration<double> wall = std::chrono::steady_clock::now() - global_start;
  std::cout << "==================================================\n";
  std::cout << "   EXECUTION COMPLETE                             \n";
  std::cout << "==================================================\n";
  std::cout << "Build Time (forest + init + NN-Descent): " << stats.build_s << "s\n";
  std::cout << "Total Execution Time: " << wall.count() << "s\n";
  return 0;
}
