// mcpgpu_cli -- C++ host program mirroring MCPNet's `mi`, `mcp`, `dpi` and
// `mcpnet` apps for the GPU method, over the mcpgpu C ABI (include/mcpgpu.hpp).
//
//   mcpgpu_cli mi     -i expr.exp -o mi.exp [-m 1] [-b 10] [-l 3] [--seed S]
//   mcpgpu_cli mcp    -i mi.exp -o mcp.exp -m {1,2,3} [--diagonal 0] [-x maxmin.exp]
//                     [-f tfs.txt [--tf-gene-transition T]] [--clamped]
//   mcpgpu_cli mcp    -i mi.exp -o mcp.exp -m 5 --first a.exp --second b.exp [--diagonal 0] [-x maxmin.exp]
//   mcpgpu_cli dpi    -i mi.exp -o dpi.exp [-l 0.1] [--diagonal 0] [-f tfs.txt]   (diagonal 0 by default)
//   mcpgpu_cli mcpnet -i expr.exp -o prefix [--mi-method 1] [--mi-input] [-m 1 2 3 4] [-f coeffs.exp]
//                     [--eval (-g truth.txt | -x truth.exp)] [--diagonal 0] [--seed S] [--tf-input tfs.txt]
//   mcpgpu_cli transform -i mi.exp -o out.exp -m {1,2} [-f tfs.txt]   (1 = CLR, 2 = Stouffer)
//   mcpgpu_cli eval_mcpnet (-i expr.exp [--mi-method 0] | --mi-file mi.exp) (-g truth.txt | -x truth.exp)
//                     [-m 1 2 3 4 5] [-f coeffs.exp] [--iterations 100] [--diagonal 0] [--tf-input tfs.txt]
//   mcpgpu_cli auc_pr_roc -i scores.exp (-g truth.txt | -x truth.exp)
//   mcpgpu_cli convert -i a.exp -o b.csv          (no GPU needed)
//
// Method values keep the reference's numbering and add the GPU forms:
//   MI  (`mi -m`, `mcpnet --mi-method`): 0 = B-spline (the reference's method;
//       here the FP32 GPU path), 1 = adaptive partitioning (the reference's
//       default; U[0, 1e-5) tie-breaking noise added first, as mi.cpp:121-131 and
//       mcpnet.cpp:293 do), 2 = B-spline on tensor cores, BF16 hi+lo split,
//       3 = BF16, 4 = FP16, 5 = FP16 hi+lo, 6 = BF16 hi*hi plus the E4M3
//       hi*lo + lo*hi correction (the fastest form within 1e-4 nats).
//   MCP (`mcp -m`, `mcpnet -m`): 1 = MCP2, 2 = MCP3, 3 = MCP4 (apps/filter/mcp.cpp:62-66),
//       and for mcpnet 4 = ensemble MCP (apps/pipeline/mcpnet.cpp:63-68, 519-719)
//       with its Stouffer variant (row statistics: see include/mcpgpu.h).
// mcp -f / dpi -f (apps/filter/mcp.cpp:94-95, dpi.cpp:80-81) keep TF rows: mcp runs
// compute_mcp{2,3,4}_tfs with --tf-gene-transition (the app's default -1 acts as 0
// for MCP2 / MCP3 and as 1 for MCP4, whose second product masks on any value but 0,
// mcp.cpp:526-537), without MCP3's max(M, M^T); dpi runs dpi_tf_kernel over all pairs
// and writes the TF rows (dpi.cpp:224-303; its --tf-gene-transition is unused).
// mcp -m 5 (MCP from partials, mcp.cpp:616-650): ratio(input, first (x) second); the app
// itself reads --first for both operands (mcp.cpp:185-195), here --second is read.
// --clamped is accepted and, as in the app, changes nothing.
// transform (apps/transform/transform.cpp): -m 1 CLR, 2 Stouffer of the square matrix with
// each row's mean and unbiased sd without its diagonal entry (GaussianParamsExclude1); with
// -f, the TF rows z-scored by row and by column (StandardScore) and combined by
// zscored_clr_kernel / zscored_stouffer_kernel (transform.cpp:156-209).
// auc_pr_roc (apps/transform/auc_pr_roc.cpp) prints `Computed,aupr <a>,,<sec>,sec` and
// `Computed,auroc <b>,,<sec>,sec` of a score matrix against the truth (list: the listed
// pairs; matrix: below the diagonal).
// eval_mcpnet (apps/pipeline/eval_mcpnet.cpp) prints the semi-supervised evaluation:
// for MI and each MCP requested, the AUPR of the labelled entries and, over
// --iterations shuffles of them (std::shuffle, std::mt19937 seeded 1, 2, ...), the
// min / max / mean / stdev of the AUPRs of the first 0.5 / 1 / 2 / 5 / 10 % (to 50 %
// with TFs) and of the rest; with -m 4 / 5 the ensemble's coefficient row chosen on
// each training part (plain and, with 5, Stouffer), summarised every 10 iterations.
// Its means divide by iterations - 1, as the app's (eval_mcpnet.cpp:307).
// mcpnet outputs follow apps/pipeline/mcpnet.cpp: <prefix>_{bs|ap|inmi}.mi.<ext>,
// .mcp2/.mcp3/.mcp4.<ext>, and for the ensemble .mcp_<c0>_<c1>_<c2>_<c3>.<ext>
// and the Stouffer-transformed .mcpst_<c0>_<c1>_<c2>_<c3>.<ext> (coefficients
// with three decimals) -- every coefficient row without --eval, the rows of
// highest AUPR with it.  <ext> is the input's (exp, csv or bin).
// --tf-input (one gene name per line; load_tfs, mcpnet_helper.hpp:1074-1123)
// restricts mcpnet to transcription-factor sources as mcpnet.cpp does: the
// prefix gets "_tf", every output has one row per TF (gene order) and all
// genes as columns -- the MI rows of the TFs, compute_mcp{2,3,4}_tfs with TF
// transitions 1 / 2 / 3, the ensemble from compute_maxmins_tfs and the TF
// Stouffer transform (compute_stouffer_tf); the truth keeps TF sources only
// (filter_list_by_tfs / filter_mat_rows_by_tfs, then select_from_list /
// select_tfs_from_mat).
// --eval prints `Computed,auprroc,<name>,<aupr>,<auroc>` per evaluated matrix:
//   -g list of "source target label" lines (label 1 / 0 / other = unknown):
//      the listed pairs of known genes, source != target (select_from_list);
//   -x label matrix (same gene order as the input): entries below the
//      diagonal (select_lower_triangle, mcpnet_helper.hpp:862-891).
// Matrix files: EXP (tab-separated "Id Alias <samples>" header, rows
// "<gene> --- <values>", the reference's text format, data/r10c10.exp), CSV
// (the same columns separated by commas; the Alias column is optional when
// reading) or raw binary ".bin" (int64 rows, int64 cols, float32 row-major).
// Genes are rows.
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <charconv>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <cmath>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "mcpgpu.hpp"

namespace {

using mcpgpu::Matrix;

struct Named {
    Matrix<float> m;
    std::vector<std::string> rows, cols;
};

bool ends_with(const std::string& s, const std::string& e) {
    return s.size() >= e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}

std::string ext_of(const std::string& path) {
    if (ends_with(path, ".bin")) return ".bin";
    if (ends_with(path, ".csv")) return ".csv";
    return ".exp";
}

std::vector<std::string> split(const std::string& line, char sep) {
    std::vector<std::string> out;
    std::stringstream ss(line);
    std::string tok;
    while (std::getline(ss, tok, sep)) {
        if (!tok.empty() && tok.back() == '\r') tok.pop_back();
        out.push_back(tok);
    }
    return out;
}

// One float token (up to the separator): std::from_chars, or strtof for what it
// does not take (a leading '+' or blank); an unparsable token reads as 0, as strtof.
float parse_float(const char* b, const char* e) {
    float v = 0.0f;
    const auto r = std::from_chars(b, e, v);
    if (r.ec == std::errc() && r.ptr != b) return v;
    const std::string tok(b, e);
    return std::strtof(tok.c_str(), nullptr);
}

Named read_matrix(const std::string& path) {
    Named r;
    if (ends_with(path, ".bin")) {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error("cannot open " + path);
        int64_t rows = 0, cols = 0;
        f.read(reinterpret_cast<char*>(&rows), 8);
        f.read(reinterpret_cast<char*>(&cols), 8);
        if (!f || rows < 0 || cols < 0) throw std::runtime_error("bad header in " + path);
        r.m = Matrix<float>(rows, cols);
        f.read(reinterpret_cast<char*>(r.m.data()), (std::streamsize)(rows * cols * 4));
        if (!f) throw std::runtime_error("truncated " + path);
        for (int64_t i = 0; i < rows; ++i) r.rows.push_back(std::to_string(i));
        for (int64_t j = 0; j < cols; ++j) r.cols.push_back(std::to_string(j));
        return r;
    }
    // Text (EXP: tab, CSV: comma): the whole file is read, its data lines located,
    // then parsed in parallel straight into the matrix rows.
    const char sep = ends_with(path, ".csv") ? ',' : '\t';
    std::FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) throw std::runtime_error("cannot open " + path);
    std::string text;
    {
        char chunk[1 << 16];
        size_t got;
        while ((got = std::fread(chunk, 1, sizeof chunk, fp)) > 0) text.append(chunk, got);
        std::fclose(fp);
    }
    // line spans [b, e) without the newline or a trailing '\r'
    std::vector<std::pair<size_t, size_t>> lines;
    for (size_t pos = 0; pos < text.size();) {
        const void* nl = std::memchr(text.data() + pos, '\n', text.size() - pos);
        size_t e = nl ? (size_t)((const char*)nl - text.data()) : text.size();
        const size_t next = nl ? e + 1 : text.size();
        if (e > pos && text[e - 1] == '\r') --e;
        if (e > pos || lines.empty()) lines.emplace_back(pos, e);  // the header may not be skipped
        pos = next;
    }
    if (lines.empty() || text.empty()) throw std::runtime_error("empty file " + path);
    std::vector<std::string> head = split(text.substr(lines[0].first, lines[0].second - lines[0].first), sep);
    const bool alias = head.size() >= 2 && head[1] == "Alias";
    const size_t skip = alias ? 2 : 1;
    for (size_t k = skip; k < head.size(); ++k) r.cols.push_back(head[k]);
    const int64_t nrows = (int64_t)lines.size() - 1, ncols = (int64_t)r.cols.size();
    r.m = Matrix<float>(nrows, ncols);
    r.rows.assign((size_t)nrows, std::string());
    int64_t bad = -1;  // the first row with the wrong number of values
#pragma omp parallel for schedule(dynamic, 64) reduction(max : bad)
    for (int64_t i = 0; i < nrows; ++i) {
        const char* p = text.data() + lines[(size_t)i + 1].first;
        const char* end = text.data() + lines[(size_t)i + 1].second;
        int64_t field = 0, nv = 0;
        float* out = r.m.data(i);
        while (true) {
            const char* q = (const char*)std::memchr(p, sep, (size_t)(end - p));
            const char* fe = q ? q : end;
            if (field == 0) {
                r.rows[(size_t)i].assign(p, fe);
            } else if (field >= (int64_t)skip) {
                if (nv < ncols) out[nv] = parse_float(p, fe);
                ++nv;
            }
            ++field;
            if (!q) break;
            p = q + 1;
        }
        if (nv != ncols) bad = std::max(bad, nrows - i);  // max of (nrows - i): the smallest i
    }
    if (bad >= 0) {
        const int64_t i = nrows - bad;
        throw std::runtime_error("row " + r.rows[(size_t)i] + " of " + path + " has the wrong number of values");
    }
    return r;
}

// Text rows are formatted in parallel blocks (std::to_chars, 9 significant digits
// as "%.9g": every float reads back exactly, also through a double) and written in
// order.
void write_matrix(const std::string& path, const Matrix<float>& m, const std::vector<std::string>& rows,
                  const std::vector<std::string>& cols) {
    if (ends_with(path, ".bin")) {
        std::ofstream f(path, std::ios::binary);
        int64_t r = m.rows(), c = m.columns();
        f.write(reinterpret_cast<const char*>(&r), 8);
        f.write(reinterpret_cast<const char*>(&c), 8);
        for (int64_t i = 0; i < r; ++i) f.write(reinterpret_cast<const char*>(m.data(i)), (std::streamsize)(c * 4));
        if (!f) throw std::runtime_error("cannot write " + path);
        return;
    }
    const char sep = ends_with(path, ".csv") ? ',' : '\t';
    std::FILE* f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::string head = std::string("Id") + sep + "Alias";
    for (int64_t j = 0; j < m.columns(); ++j) {
        head += sep;
        head += j < (int64_t)cols.size() ? cols[(size_t)j] : std::to_string(j);
    }
    head += '\n';
    bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
    const int64_t R = m.rows(), C = m.columns();
    const int64_t per_block = std::max<int64_t>(1, (int64_t)(8 << 20) / std::max<int64_t>(1, C * 16));  // ~8 MB
    const int64_t blocks = (R + per_block - 1) / per_block;
#pragma omp parallel
    {
        std::string buf;
#pragma omp for ordered schedule(static, 1)
        for (int64_t b = 0; b < blocks; ++b) {
            buf.clear();
            char num[32];
            for (int64_t i = b * per_block; i < std::min(R, (b + 1) * per_block); ++i) {
                buf += i < (int64_t)rows.size() ? rows[(size_t)i] : std::to_string(i);
                buf += sep;
                buf += "---";
                const float* row = m.data(i);
                for (int64_t j = 0; j < C; ++j) {
                    const auto res = std::to_chars(num, num + sizeof num, row[j], std::chars_format::general, 9);
                    buf += sep;
                    buf.append(num, res.ptr);
                }
                buf += '\n';
            }
#pragma omp ordered
            if (std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) ok = false;
        }
    }
    if (std::fclose(f) != 0 || !ok) throw std::runtime_error("cannot write " + path);
}

struct Args {
    std::string cmd, in, out, maxmin_out, coeffs, truth_list, truth_mat, tf_input, first, second, mi_file;
    int bins = 10, order = 3, mi_method = -1, tf_transition = -1;
    int64_t iterations = 100;
    std::vector<int> methods;
    float diagonal = 0.0f, tol = 0.1f;
    uint64_t seed = 1;
    bool diagonal_set = false, mi_input = false, eval = false;
};

Args parse(int argc, char** argv) {
    Args a;
    if (argc < 2)
        throw std::runtime_error(
            "usage: mcpgpu_cli {mi|mcp|dpi|mcpnet|eval_mcpnet|transform|auc_pr_roc|convert} -i IN [-o OUT] [options]");
    a.cmd = argv[1];
    for (int i = 2; i < argc; ++i) {
        std::string k = argv[i];
        auto next = [&]() -> std::string {
            if (i + 1 >= argc) throw std::runtime_error("missing value after " + k);
            return argv[++i];
        };
        if (k == "-i" || k == "--input") a.in = next();
        else if (k == "-o" || k == "--output") a.out = next();
        else if (k == "-b" || k == "--bins") a.bins = std::atoi(next().c_str());
        else if (k == "--spline_order") a.order = std::atoi(next().c_str());
        else if (k == "-l" || k == "--tolerance") {
            std::string v = next();
            if (a.cmd == "mi") a.order = std::atoi(v.c_str());  // mi -l = spline order
            else a.tol = std::strtof(v.c_str(), nullptr);
        } else if (k == "--mi-method") a.mi_method = std::atoi(next().c_str());
        else if (k == "--mi-input") a.mi_input = true;
        else if (k == "-m" || k == "--method") {
            a.methods.push_back(std::atoi(next().c_str()));
            while (i + 1 < argc && argv[i + 1][0] != '-') a.methods.push_back(std::atoi(argv[++i]));
        } else if (k == "--diagonal") {
            a.diagonal = std::strtof(next().c_str(), nullptr);
            a.diagonal_set = true;
        } else if (k == "-x") {
            if (a.cmd == "mcp") a.maxmin_out = next();  // mcp -x = max-min output
            else a.truth_mat = next();                  // mcpnet -x = truth matrix
        } else if (k == "--maxmin-output") a.maxmin_out = next();
        else if (k == "--groundtruth-matrix") a.truth_mat = next();
        else if (k == "-g" || k == "--groundtruth-list") a.truth_list = next();
        else if (k == "-f") {
            if (a.cmd == "mcpnet" || a.cmd == "eval_mcpnet") a.coeffs = next();  // -f = coefficients there
            else a.tf_input = next();                  // mcp / dpi -f = TF list
        } else if (k == "--coefficients") a.coeffs = next();
        else if (k == "--tf-gene-transition") a.tf_transition = std::atoi(next().c_str());
        else if (k == "--first") a.first = next();
        else if (k == "--second") a.second = next();
        else if (k == "--clamped" || k == "--permute-combo") {}  // no effect, as in the apps
        else if (k == "--iterations") a.iterations = std::atoll(next().c_str());
        else if (k == "--mi-file") a.mi_file = next();
        else if (k == "--eval") a.eval = true;
        else if (k == "--seed") a.seed = std::strtoull(next().c_str(), nullptr, 10);
        else if (k == "--tf-input") a.tf_input = next();
        else throw std::runtime_error("unknown option " + k);
    }
    if (a.cmd == "auc_pr_roc") {
        if (a.in.empty()) throw std::runtime_error("auc_pr_roc needs -i (score matrix)");
        if (a.truth_list.empty() == a.truth_mat.empty())
            throw std::runtime_error("auc_pr_roc needs exactly one of -g (truth list) and -x (truth matrix)");
        a.eval = true;
        return a;
    }
    if (a.cmd == "eval_mcpnet") {
        if (a.in.empty() == a.mi_file.empty())
            throw std::runtime_error("eval_mcpnet needs exactly one of -i (expression) and --mi-file");
        if (a.truth_list.empty() == a.truth_mat.empty())
            throw std::runtime_error("eval_mcpnet needs exactly one of -g (truth list) and -x (truth matrix)");
        if (a.iterations < 0) throw std::runtime_error("--iterations must be >= 0");
        a.eval = true;
        return a;
    }
    if (a.in.empty() || a.out.empty()) throw std::runtime_error("-i and -o are required");
    if (a.eval && a.truth_list.empty() == a.truth_mat.empty())
        throw std::runtime_error("--eval needs exactly one of -g (truth list) and -x (truth matrix)");
    return a;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// MI by method number; returns the output-name tag of the method.
std::string compute_mi(mcpgpu::Context& ctx, const Named& in, int method, int bins, int order, uint64_t seed,
                       Matrix<float>& mi) {
    switch (method) {
        case 0: mcpgpu::compute_mi(ctx, in.m, bins, mi, mcpgpu::MIPrecision::FP32, order); return "_bs";
        case 1: mcpgpu::compute_ap_mi(ctx, in.m, mi, true, seed); return "_ap";
        case 2: mcpgpu::compute_mi(ctx, in.m, bins, mi, mcpgpu::MIPrecision::BF16X3, order); return "_bs";
        case 3: mcpgpu::compute_mi(ctx, in.m, bins, mi, mcpgpu::MIPrecision::BF16, order); return "_bs";
        case 4: mcpgpu::compute_mi(ctx, in.m, bins, mi, mcpgpu::MIPrecision::FP16, order); return "_bs";
        case 5: mcpgpu::compute_mi(ctx, in.m, bins, mi, mcpgpu::MIPrecision::FP16X3, order); return "_bs";
        case 6: mcpgpu::compute_mi(ctx, in.m, bins, mi, mcpgpu::MIPrecision::BF16F8, order); return "_bs";
        default:
            throw std::runtime_error("unsupported MI method " + std::to_string(method) +
                                     " (0 = B-spline FP32, 1 = adaptive partitioning, 2..6 = tensor-core B-spline)");
    }
}

std::string trim(const std::string& s) {
    const char* ws = " \t\r\n\f\v";
    const size_t b = s.find_first_not_of(ws);
    if (b == std::string::npos) return "";
    return s.substr(b, s.find_last_not_of(ws) - b + 1);
}

// The TF selection of --tf-input (load_tfs, mcpnet_helper.hpp:1074-1123).
struct TfSel {
    bool on = false;
    std::vector<float> tfs;         // per gene: +inf for a TF, -inf otherwise
    std::vector<int32_t> rows;      // gene index of every TF, in gene order
    std::vector<uint8_t> col_tf;    // per gene: 1 for a TF
    std::vector<std::string> names;
};

TfSel load_tfs(const std::string& path, const std::vector<std::string>& genes) {
    TfSel t;
    if (path.empty()) return t;
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::set<std::string> names;
    std::string line;
    while (std::getline(f, line)) names.insert(trim(line));
    t.on = true;
    for (size_t i = 0; i < genes.size(); ++i) {
        const bool tf = names.count(trim(genes[i])) > 0;
        t.tfs.push_back(tf ? INFINITY : -INFINITY);
        t.col_tf.push_back(tf ? 1 : 0);
        if (tf) {
            t.rows.push_back((int32_t)i);
            t.names.push_back(genes[i]);
        }
    }
    return t;
}

// Truth labels over the output matrix (genes x genes, or TFs x genes) and the
// region they are read from.
struct Truth {
    Matrix<int8_t> labels;
    mcpgpu::TruthRegion region = mcpgpu::TruthRegion::LowerTriangle;
    const TfSel* tf = nullptr;
};

Truth read_truth(const Args& a, const std::vector<std::string>& genes, const TfSel& tf) {
    Truth t;
    const int64_t n = (int64_t)genes.size();
    const int64_t rows = tf.on ? (int64_t)tf.rows.size() : n;
    t.labels = Matrix<int8_t>(rows, n);
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < n; ++j) t.labels.at(i, j) = -1;
    if (!a.truth_list.empty()) {
        // read_groundtruth + select_from_list (mcpnet_helper.hpp:641-668, 840-859); with TFs only
        // the pairs whose source is a TF (filter_list_by_tfs, mcpnet_helper.hpp:1173-1193)
        std::map<std::string, int64_t> src, id;
        for (int64_t i = 0; i < n; ++i) id[genes[(size_t)i]] = i;
        if (tf.on)
            for (int64_t r = 0; r < rows; ++r) src[tf.names[(size_t)r]] = r;
        else
            src = id;
        std::ifstream f(a.truth_list);
        if (!f) throw std::runtime_error("cannot open " + a.truth_list);
        std::string s, d;
        int g;
        while (f >> s >> d >> g) {
            if (s == d) continue;
            auto is = src.find(s), it = id.find(d);
            if (is == src.end() || it == id.end()) continue;
            t.labels.at(is->second, it->second) = (int8_t)((g == 1 || g == 0) ? g : -1);
        }
        t.region = mcpgpu::TruthRegion::All;
    } else {
        Named m = read_matrix(a.truth_mat);
        if (m.m.rows() != n || m.m.columns() != n)
            throw std::runtime_error("truth matrix is " + std::to_string(m.m.rows()) + " x " +
                                     std::to_string(m.m.columns()) + ", expected " + std::to_string(n) + " x " +
                                     std::to_string(n));
        // with TFs: its TF rows (filter_mat_rows_by_tfs) and select_tfs_from_mat's region
        for (int64_t i = 0; i < rows; ++i)
            for (int64_t j = 0; j < n; ++j) {
                const float v = m.m.at(tf.on ? tf.rows[(size_t)i] : i, j);
                t.labels.at(i, j) = (int8_t)(v == 1.0f ? 1 : v == 0.0f ? 0 : -1);
            }
        t.region = tf.on ? mcpgpu::TruthRegion::TFRows : mcpgpu::TruthRegion::LowerTriangle;
    }
    t.tf = tf.on ? &tf : nullptr;
    return t;
}

void report(mcpgpu::Context& ctx, const Truth& t, const Matrix<float>& values, const std::string& name) {
    mcpgpu::Curves c = mcpgpu::compute_aupr_auroc(ctx, t.labels, values, t.region, t.tf ? &t.tf->rows : nullptr,
                                                  t.tf ? &t.tf->col_tf : nullptr);
    std::printf("Computed,auprroc,%s,%.12g,%.12g,pos=%lld,neg=%lld\n", name.c_str(), c.aupr, c.auroc,
                (long long)c.n_pos, (long long)c.n_neg);
}

std::string coeff_tag(const double* c) {
    char b[128];
    std::snprintf(b, sizeof b, "%.3f_%.3f_%.3f_%.3f", c[0], c[1], c[2], c[3]);
    return b;
}

std::vector<double> read_coeffs(const std::string& path) {
    std::vector<double> cs;
    if (path.empty()) return {0.25, 0.25, 0.25, 0.25};  // mcpnet.cpp:533-539
    if (ends_with(path, ".exp") || ends_with(path, ".csv") || ends_with(path, ".bin")) {
        Named m = read_matrix(path);
        if (m.m.columns() != 4) throw std::runtime_error("coefficient file must have 4 columns");
        for (int64_t i = 0; i < m.m.rows(); ++i)
            for (int64_t j = 0; j < 4; ++j) cs.push_back(m.m.at(i, j));
        return cs;
    }
    std::ifstream f(path);  // plain text: 4 numbers per row
    if (!f) throw std::runtime_error("cannot open " + path);
    double v;
    while (f >> v) cs.push_back(v);
    if (cs.empty() || cs.size() % 4) throw std::runtime_error("coefficient file must hold rows of 4 numbers");
    return cs;
}

// Per part: min, max, sum and sum of squares of the AUPRs seen so far
// (eval_mcpnet.cpp:255-300: min starts at DBL_MAX, the rest at 0).
struct PartStats {
    std::vector<double> s;
    explicit PartStats(size_t parts) : s(4 * parts, 0.0) {
        for (size_t j = 0; j < parts; ++j) s[4 * j] = DBL_MAX;
    }
    void add(size_t j, double a) {
        s[4 * j] = std::min(s[4 * j], a);
        s[4 * j + 1] = std::max(s[4 * j + 1], a);
        s[4 * j + 2] += a;
        s[4 * j + 3] += a * a;
    }
    // the app's lines (eval_mcpnet.cpp:305-317); its mean divides by i - 1
    void print(const std::string& what, size_t j, int64_t i) const {
        const double n = (double)i;
        const double mean = s[4 * j + 2] / n;
        const double sd = std::sqrt(n / (n - 1.0) * (s[4 * j + 3] / n - mean * mean));
        std::printf("AUPR %s min,%.12g,decile %zu,iters %lld,sec\n", what.c_str(), s[4 * j], j, (long long)i);
        std::printf("AUPR %s max,%.12g,decile %zu,iters %lld,sec\n", what.c_str(), s[4 * j + 1], j, (long long)i);
        std::printf("AUPR %s mean,%.12g,decile %zu,iters %lld,sec\n", what.c_str(), s[4 * j + 2] / (n - 1.0), j,
                    (long long)i);
        std::printf("AUPR %s stdev,%.12g,decile %zu,iters %lld,sec\n", what.c_str(), sd, j, (long long)i);
    }
};

// eval_aupr_mcp (eval_mcpnet.cpp:227-317) of one score matrix.
void report_split(mcpgpu::Context& ctx, const Truth& t, const Matrix<float>& values, int64_t iterations,
                  const std::string& tag) {
    const mcpgpu::Curves c = mcpgpu::compute_aupr_auroc(ctx, t.labels, values, t.region,
                                                       t.tf ? &t.tf->rows : nullptr, t.tf ? &t.tf->col_tf : nullptr);
    const int64_t E = c.n_pos + c.n_neg;  // the labelled entries
    const std::vector<int64_t> counts = mcpgpu::train_counts(E, t.tf != nullptr);
    mcpgpu::SplitAupr r = mcpgpu::split_aupr(ctx, t.labels, values, iterations, counts, t.region,
                                             t.tf ? &t.tf->rows : nullptr, t.tf ? &t.tf->col_tf : nullptr);
    std::printf("AUPR %s,%.12g,,,sec\n", tag.c_str(), r.full);
    const size_t parts = counts.size();
    PartStats tr(parts), te(parts);
    for (int64_t i = 0; i < iterations; ++i)
        for (size_t j = 0; j < parts; ++j) {
            tr.add(j, r.train[(size_t)i * parts + j]);
            te.add(j, r.test[(size_t)i * parts + j]);
        }
    for (size_t j = 0; j < parts; ++j) {
        tr.print(tag + " train", j, iterations);
        te.print(tag + " test", j, iterations);
    }
}

}  // namespace

int main(int argc, char** argv) {
    try {
        Args a = parse(argc, argv);
        Named in = read_matrix(a.in.empty() ? a.mi_file : a.in);
        double t0 = now_s();
        if (a.cmd == "convert") {
            write_matrix(a.out, in.m, in.rows, in.cols);
            return 0;
        }
        // the TF list is checked before the device is touched (mcpnet.cpp:207-211)
        const TfSel tf = a.cmd == "convert" ? TfSel{} : load_tfs(a.tf_input, in.rows);
        if (tf.on && tf.rows.empty()) {
            std::fprintf(stderr, "ERROR: no transcription factors in the specified file\n");
            return 1;
        }
        mcpgpu::Context ctx(0);
        if (a.cmd == "mi") {
            int method = a.methods.empty() ? 1 : a.methods[0];
            Matrix<float> mi;
            compute_mi(ctx, in, method, a.bins, a.order, a.seed, mi);
            std::printf("Computed,MI,,%.6f,sec\n", now_s() - t0);
            write_matrix(a.out, mi, in.rows, in.rows);
        } else if (a.cmd == "mcp") {
            int method = a.methods.empty() ? 1 : a.methods[0];
            if (method != 5 && (method < 1 || method > 3))
                throw std::runtime_error("mcp -m must be 1 (MCP2), 2 (MCP3), 3 (MCP4) or 5 (MCP from partials)");
            if (a.diagonal_set) mcpgpu::set_diagonal(in.m, a.diagonal);  // the mcp app resets only on request
            Matrix<float> ratio, maxmin;
            if (method == 5) {  // MCP from partials (mcp.cpp:616-650)
                if (tf.on) throw std::runtime_error("transcription factors are not supported with mcp -m 5");
                if (a.first.empty() || a.second.empty()) throw std::runtime_error("mcp -m 5 needs --first and --second");
                Named f1 = read_matrix(a.first), f2 = read_matrix(a.second);
                if (a.diagonal_set) {
                    mcpgpu::set_diagonal(f1.m, a.diagonal);
                    mcpgpu::set_diagonal(f2.m, a.diagonal);
                }
                if (f1.m.columns() != f2.m.columns() || f1.m.rows() != in.m.rows() || f2.m.rows() != in.m.columns())
                    throw std::runtime_error("mcp -m 5: --first must be n x k and --second n x k for an n x n input");
                mcpgpu::maxmin(ctx, f1.m, f2.m, maxmin);
                mcpgpu::compute_ratio(ctx, in.m, maxmin, ratio);
            } else if (tf.on) {
                // the app's default transition -1 (mcp.cpp:77) takes the branches of 0 for MCP2 / MCP3 and of 1 for
                // MCP4 (its second product is masked for every value but 0)
                int tr = a.tf_transition;
                if (tr < 0) tr = method == 3 ? 1 : 0;
                mcpgpu::compute_mcp_tfs(ctx, in.m, tf.tfs, method + 1, tr, ratio, &maxmin);
            } else {
                // the mcp app symmetrises MCP3 (apps/filter/mcp.cpp:463-476)
                mcpgpu::compute_mcp(ctx, in.m, method + 1, ratio, &maxmin, method == 2);
            }
            std::printf("Compute MCP%d in %.6f sec\n", method == 5 ? 2 : method + 1, now_s() - t0);
            const std::vector<std::string>& rn = tf.on ? tf.names : in.rows;
            if (!a.maxmin_out.empty()) write_matrix(a.maxmin_out, maxmin, rn, in.rows);
            write_matrix(a.out, ratio, rn, in.rows);
        } else if (a.cmd == "dpi") {
            mcpgpu::set_diagonal(in.m, a.diagonal);
            Matrix<float> out;
            int64_t removed = tf.on ? mcpgpu::dpi_filter_tfs(ctx, in.m, a.tol, tf.tfs, out)
                                    : mcpgpu::dpi_filter(ctx, in.m, a.tol, out);
            std::printf("Mask removing %lld elements \n", (long long)removed);
            if (tf.on) {  // keep the TF rows (dpi.cpp:292-303)
                Matrix<float> rows((int64_t)tf.rows.size(), out.columns());
                for (size_t r = 0; r < tf.rows.size(); ++r)
                    for (int64_t j = 0; j < out.columns(); ++j) rows.at((int64_t)r, j) = out.at(tf.rows[r], j);
                write_matrix(a.out, rows, tf.names, in.rows);
            } else {
                write_matrix(a.out, out, in.rows, in.rows);
            }
        } else if (a.cmd == "transform") {
            int method = a.methods.empty() ? 2 : a.methods[0];
            if (method != 1 && method != 2) throw std::runtime_error("transform -m must be 1 (CLR) or 2 (Stouffer)");
            if (in.m.rows() != in.m.columns()) throw std::runtime_error("transform needs a square matrix");
            Matrix<float> out;
            if (tf.on) {
                Matrix<float> rows((int64_t)tf.rows.size(), in.m.columns());
                for (size_t r = 0; r < tf.rows.size(); ++r)
                    for (int64_t j = 0; j < in.m.columns(); ++j) rows.at((int64_t)r, j) = in.m.at(tf.rows[r], j);
                mcpgpu::compute_stouffer_tf(ctx, rows, out, method == 1);
            } else {
                mcpgpu::compute_stouffer(ctx, in.m, out, method == 1);
            }
            std::printf("Transformed in %.6f sec\n", now_s() - t0);
            write_matrix(a.out, out, tf.on ? tf.names : in.rows, in.rows);
        } else if (a.cmd == "auc_pr_roc") {  // apps/transform/auc_pr_roc.cpp:380-460
            if (in.m.rows() != in.m.columns()) throw std::runtime_error("auc_pr_roc needs a square score matrix");
            const Truth truth = read_truth(a, in.rows, tf);
            const double t1 = now_s();
            const mcpgpu::Curves c = mcpgpu::compute_aupr_auroc(ctx, truth.labels, in.m, truth.region);
            const double dt = now_s() - t1;
            std::printf("Computed,aupr %.12g,,%.6f,sec\n", c.aupr, dt);
            std::printf("Computed,auroc %.12g,,%.6f,sec\n", c.auroc, dt);
        } else if (a.cmd == "eval_mcpnet") {  // apps/pipeline/eval_mcpnet.cpp:464-893
            const std::vector<std::string>& genes = in.rows;
            Truth truth = read_truth(a, genes, tf);
            Matrix<float> mi;
            if (!a.mi_file.empty()) {
                if (in.m.rows() != in.m.columns()) throw std::runtime_error("--mi-file needs a square MI matrix");
                mi = in.m;
            } else {  // the app's default MI method is B-spline
                compute_mi(ctx, in, a.mi_method < 0 ? 0 : a.mi_method, a.bins, a.order, a.seed, mi);
                std::printf("Computed,MI,,%.6f,sec\n", now_s() - t0);
            }
            mcpgpu::set_diagonal(mi, a.diagonal);
            Matrix<float> mi_tf;
            if (tf.on) {
                mi_tf = Matrix<float>((int64_t)tf.rows.size(), mi.columns());
                for (size_t r = 0; r < tf.rows.size(); ++r)
                    for (int64_t j = 0; j < mi.columns(); ++j) mi_tf.at((int64_t)r, j) = mi.at(tf.rows[r], j);
            }
            const std::string tag = tf.on ? "TF" : "full";
            const Matrix<float>& base = tf.on ? mi_tf : mi;
            report_split(ctx, truth, base, a.iterations, tag);
            bool ens = false, with_st = false;
            for (int method : a.methods) {
                if (method < 1 || method > 5) throw std::runtime_error("eval_mcpnet -m accepts 1, 2, 3, 4, 5");
                if (method >= 4) {
                    ens = true;
                    with_st |= method == 5;
                    continue;
                }
                Matrix<float> ratio;
                if (tf.on) mcpgpu::compute_mcp_tfs(ctx, mi, tf.tfs, method + 1, method, ratio);
                else mcpgpu::compute_mcp(ctx, mi, method + 1, ratio);
                std::printf("Computed,MCP%d,,%.6f,sec\n", method + 1, now_s() - t0);
                report_split(ctx, truth, ratio, a.iterations, tag);
            }
            if (ens) {  // eval_combos over the splits (eval_mcpnet.cpp:737-893)
                std::vector<double> cs = read_coeffs(a.coeffs);
                Matrix<float> m1, m2, m3;
                if (tf.on) mcpgpu::compute_maxmins_tfs(ctx, mi, tf.tfs, mi_tf, m1, m2, m3);
                else mcpgpu::compute_maxmins(ctx, mi, m1, m2, m3);
                const mcpgpu::Curves c = mcpgpu::compute_aupr_auroc(ctx, truth.labels, base, truth.region,
                                                                   tf.on ? &tf.rows : nullptr,
                                                                   tf.on ? &tf.col_tf : nullptr);
                const std::vector<int64_t> counts = mcpgpu::train_counts(c.n_pos + c.n_neg, tf.on);
                const int st = !with_st ? MCPG_STOUFFER_NONE
                                        : (tf.on ? MCPG_STOUFFER_TF : MCPG_ROWSTATS_EXCLUDE_DIAGONAL);
                std::vector<double> res = mcpgpu::split_combo_eval(ctx, base, m1, m2, m3, truth.labels, cs, st,
                                                                   a.iterations, counts, truth.region,
                                                                   tf.on ? &tf.rows : nullptr,
                                                                   tf.on ? &tf.col_tf : nullptr);
                const size_t parts = counts.size();
                const char* names[6] = {"train", "test", "train", "test", "full", "full"};
                std::vector<PartStats> stats(6, PartStats(parts));
                for (int64_t i = 1; i <= a.iterations; ++i) {
                    for (size_t j = 0; j < parts; ++j)
                        for (int q = 0; q < 6; ++q) stats[(size_t)q].add(j, res[(((size_t)i - 1) * parts + j) * 6 + q]);
                    if (i % 10) continue;  // the app reports every 10 iterations
                    for (size_t j = 0; j < parts; ++j)
                        for (int q : {0, 1, 2, 3, 4, 5})
                            stats[(size_t)q].print(std::string(q == 2 || q == 3 || q == 5 ? "stouffer " : "") + tag +
                                                       " " + names[q],
                                                   j, i);
                }
            }
            std::printf("eval_mcpnet done in %.6f sec\n", now_s() - t0);
        } else if (a.cmd == "mcpnet") {
            const std::string ext = ext_of(a.in);
            const std::vector<std::string>& genes = in.rows;
            if (tf.on) std::printf("TFs specified, found %zu\n", tf.rows.size());
            const std::vector<std::string>& row_names = tf.on ? tf.names : genes;
            Truth truth;
            if (a.eval) truth = read_truth(a, genes, tf);
            Matrix<float> mi;
            std::string prefix = a.out + (tf.on ? "_tf" : "");
            if (a.mi_input) {
                if (in.m.rows() != in.m.columns()) throw std::runtime_error("--mi-input needs a square MI matrix");
                mi = in.m;
                prefix += "_inmi";
            } else {
                prefix += compute_mi(ctx, in, a.mi_method < 0 ? 1 : a.mi_method, a.bins, a.order, a.seed, mi);
                std::printf("Computed,MI,,%.6f,sec\n", now_s() - t0);
            }
            mcpgpu::set_diagonal(mi, a.diagonal);  // mcpnet.cpp:299-308 (negative: keep)
            Matrix<float> mi_tf;  // the TF rows (filter_local_mat_rows_by_tfs, mcpnet.cpp:317-325)
            if (tf.on) {
                mi_tf = Matrix<float>((int64_t)tf.rows.size(), mi.columns());
                for (size_t r = 0; r < tf.rows.size(); ++r)
                    for (int64_t j = 0; j < mi.columns(); ++j) mi_tf.at((int64_t)r, j) = mi.at(tf.rows[r], j);
            }
            const Matrix<float>& mi_out = tf.on ? mi_tf : mi;
            if (a.eval) report(ctx, truth, mi_out, "mi");
            if (!a.mi_input) write_matrix(prefix + ".mi" + ext, mi_out, row_names, genes);
            std::vector<int> ms = a.methods.empty() ? std::vector<int>{1} : a.methods;
            for (int method : ms) {
                if (method < 1 || method > 4) throw std::runtime_error("mcpnet -m accepts 1, 2, 3, 4");
                double t1 = now_s();
                if (method <= 3) {
                    Matrix<float> ratio;
                    if (tf.on) mcpgpu::compute_mcp_tfs(ctx, mi, tf.tfs, method + 1, method, ratio);  // mcpnet.cpp:377,428,475
                    else mcpgpu::compute_mcp(ctx, mi, method + 1, ratio);
                    std::printf("Computed,MCP%d,,%.6f,sec\n", method + 1, now_s() - t1);
                    if (a.eval) report(ctx, truth, ratio, "mcp" + std::to_string(method + 1));
                    write_matrix(prefix + ".mcp" + std::to_string(method + 1) + ext, ratio, row_names, genes);
                    continue;
                }
                // ensemble MCP (mcpnet.cpp:519-719)
                std::vector<double> cs = read_coeffs(a.coeffs);
                Matrix<float> m1, m2, m3, combo;
                if (tf.on) mcpgpu::compute_maxmins_tfs(ctx, mi, tf.tfs, mi_tf, m1, m2, m3);
                else mcpgpu::compute_maxmins(ctx, mi, m1, m2, m3);
                std::printf("Computed,MAXMIN 1 2 3,,%.6f,sec\n", now_s() - t1);
                const Matrix<float>& base = tf.on ? mi_tf : mi;
                auto stouffer = [&](const Matrix<float>& c, Matrix<float>& st) {
                    if (tf.on) mcpgpu::compute_stouffer_tf(ctx, c, st);  // mcpnet.cpp:623-628
                    else mcpgpu::compute_stouffer(ctx, c, st);
                };
                const int64_t nc = (int64_t)(cs.size() / 4);
                if (a.eval) {
                    const std::vector<int32_t>* rg = tf.on ? &tf.rows : nullptr;
                    const std::vector<uint8_t>* ct = tf.on ? &tf.col_tf : nullptr;
                    std::vector<double> pr, roc;
                    int64_t best = mcpgpu::select_combo(ctx, base, m1, m2, m3, truth.labels, cs, &pr, &roc,
                                                        truth.region, rg, ct);
                    for (int64_t c = 0; c < nc; ++c)
                        if (pr[(size_t)c] == pr[(size_t)c])  // rows (1,0,0,0) are skipped (NaN)
                            std::printf("Computed,Combo AUPR %.12g,(%s),AUROC %.12g\n", pr[(size_t)c],
                                        coeff_tag(&cs[(size_t)(4 * c)]).c_str(), roc[(size_t)c]);
                    const double* c = &cs[(size_t)(4 * best)];
                    mcpgpu::compute_combo(ctx, base, m1, m2, m3, c, combo);
                    std::printf("Computed,MAX Combo aupr %.12g,(%s)\n", pr[(size_t)best], coeff_tag(c).c_str());
                    write_matrix(prefix + ".mcp_" + coeff_tag(c) + ext, combo, row_names, genes);
                    // the Stouffer half (mcpnet.cpp:622-661, 691-708)
                    std::vector<double> spr, sroc;
                    int64_t sbest =
                        tf.on ? mcpgpu::select_combo_stouffer_tf(ctx, base, m1, m2, m3, truth.labels, cs, &spr, &sroc,
                                                                 truth.region, rg, ct)
                              : mcpgpu::select_combo_stouffer(ctx, base, m1, m2, m3, truth.labels, cs, &spr, &sroc,
                                                              truth.region);
                    for (int64_t r = 0; r < nc; ++r)
                        if (spr[(size_t)r] == spr[(size_t)r])
                            std::printf("Computed,Combo Stouffer AUPR %.12g,(%s),AUROC %.12g\n", spr[(size_t)r],
                                        coeff_tag(&cs[(size_t)(4 * r)]).c_str(), sroc[(size_t)r]);
                    const double* sc = &cs[(size_t)(4 * sbest)];
                    Matrix<float> st;
                    mcpgpu::compute_combo(ctx, base, m1, m2, m3, sc, combo);
                    stouffer(combo, st);
                    std::printf("Computed,MAX Combo AND Stouffer aupr %.12g,(%s)\n", spr[(size_t)sbest],
                                coeff_tag(sc).c_str());
                    write_matrix(prefix + ".mcpst_" + coeff_tag(sc) + ext, st, row_names, genes);
                } else {
                    Matrix<float> st;
                    for (int64_t r = 0; r < nc; ++r) {
                        const double* c = &cs[(size_t)(4 * r)];
                        if (c[0] == 1 && c[1] == 0 && c[2] == 0 && c[3] == 0) continue;  // mcpnet.cpp:589
                        mcpgpu::compute_combo(ctx, base, m1, m2, m3, c, combo);
                        write_matrix(prefix + ".mcp_" + coeff_tag(c) + ext, combo, row_names, genes);
                        stouffer(combo, st);
                        write_matrix(prefix + ".mcpst_" + coeff_tag(c) + ext, st, row_names, genes);
                    }
                }
                std::printf("ALL Combos in %.6f sec\n", now_s() - t1);
            }
        } else {
            throw std::runtime_error("unknown command " + a.cmd);
        }
        return 0;
    } catch (const mcpgpu::Error& e) {
        std::fprintf(stderr, "mcpgpu error %d: %s\n", e.status(), e.what());
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
