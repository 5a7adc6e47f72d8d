// mcpgpu_cli -- C++ host program mirroring MCPNet's `mi`, `mcp`, `dpi` and
// `mcpnet` apps for the GPU method, over the mcpgpu C ABI (include/mcpgpu.hpp).
//
//   mcpgpu_cli mi     -i expr.exp -o mi.exp [-b 10] [-l 3] [-m 2]
//   mcpgpu_cli mcp    -i mi.exp -o mcp.exp -m {1,2,3} [--diagonal 0] [-x maxmin.exp]
//   mcpgpu_cli dpi    -i mi.exp -o dpi.exp [-l 0.1] [--diagonal 0]     (diagonal 0 by default)
//   mcpgpu_cli mcpnet -i expr.exp -o prefix [--mi-method 2] [-m 1 2 3] [--diagonal 0]
//   mcpgpu_cli convert -i a.exp -o b.bin          (no GPU needed)
//
// Method values keep the reference's numbering and add the GPU forms:
//   MI  (`mi -m`, `mcpnet --mi-method`): 0 = B-spline (the reference's CPU
//       method; here the FP32 GPU path), 2 = B-spline on tensor cores, BF16 hi+lo
//       split (default), 3 = BF16, 4 = FP16, 5 = FP16 hi+lo.
//   MCP (`mcp -m`, `mcpnet -m`): 1 = MCP2, 2 = MCP3, 3 = MCP4, as
//       apps/filter/mcp.cpp:62-66 and apps/pipeline/mcpnet.cpp:63-68.
// Matrix files: EXP (tab-separated "Id Alias <samples>" header, rows
// "<gene> --- <values>", the reference's text format, data/r10c10.exp) or raw
// binary ".bin" (int64 rows, int64 cols, float32 row-major).  Genes are rows;
// a samples-by-genes EXP is not transposed (as the reference does when the
// header names match) -- pass genes as rows.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
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
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::string line;
    if (!std::getline(f, line)) throw std::runtime_error("empty file " + path);
    {
        std::stringstream ss(line);
        std::string tok;
        std::getline(ss, tok, '\t');  // Id
        std::getline(ss, tok, '\t');  // Alias
        while (std::getline(ss, tok, '\t')) r.cols.push_back(tok);
    }
    std::vector<float> vals;
    while (std::getline(f, line)) {
        if (line.empty()) continue;
        std::stringstream ss(line);
        std::string tok;
        std::getline(ss, tok, '\t');
        r.rows.push_back(tok);
        std::getline(ss, tok, '\t');  // alias
        size_t c = 0;
        while (std::getline(ss, tok, '\t')) {
            vals.push_back(std::strtof(tok.c_str(), nullptr));
            ++c;
        }
        if (c != r.cols.size()) throw std::runtime_error("row " + r.rows.back() + " has the wrong number of values");
    }
    r.m = Matrix<float>((int64_t)r.rows.size(), (int64_t)r.cols.size());
    std::memcpy(r.m.data(), vals.data(), vals.size() * sizeof(float));
    return r;
}

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
    std::FILE* f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::fprintf(f, "Id\tAlias");
    for (int64_t j = 0; j < m.columns(); ++j)
        std::fprintf(f, "\t%s", j < (int64_t)cols.size() ? cols[(size_t)j].c_str() : std::to_string(j).c_str());
    std::fprintf(f, "\n");
    for (int64_t i = 0; i < m.rows(); ++i) {
        std::fprintf(f, "%s\t---", i < (int64_t)rows.size() ? rows[(size_t)i].c_str() : std::to_string(i).c_str());
        for (int64_t j = 0; j < m.columns(); ++j) std::fprintf(f, "\t%.9g", (double)m.at(i, j));
        std::fprintf(f, "\n");
    }
    std::fclose(f);
}

struct Args {
    std::string cmd, in, out, maxmin_out;
    int bins = 10, order = 3, mi_method = 2;
    std::vector<int> methods;
    float diagonal = 0.0f, tol = 0.1f;
    bool order_set = false, diagonal_set = false;
};

Args parse(int argc, char** argv) {
    Args a;
    if (argc < 2) throw std::runtime_error("usage: mcpgpu_cli {mi|mcp|dpi|mcpnet|convert} -i IN -o OUT [options]");
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
        else if (k == "--spline_order") { a.order = std::atoi(next().c_str()); a.order_set = true; }
        else if (k == "-l" || k == "--tolerance") {
            std::string v = next();
            if (a.cmd == "mi") { a.order = std::atoi(v.c_str()); a.order_set = true; }  // mi -l = spline order
            else a.tol = std::strtof(v.c_str(), nullptr);
        } else if (k == "--mi-method") a.mi_method = std::atoi(next().c_str());
        else if (k == "-m" || k == "--method") {
            a.methods.push_back(std::atoi(next().c_str()));
            while (i + 1 < argc && argv[i + 1][0] != '-') a.methods.push_back(std::atoi(argv[++i]));
        } else if (k == "--diagonal") {
            a.diagonal = std::strtof(next().c_str(), nullptr);
            a.diagonal_set = true;
        }
        else if (k == "-x" || k == "--maxmin-output") a.maxmin_out = next();
        else throw std::runtime_error("unknown option " + k);
    }
    if (a.in.empty() || a.out.empty()) throw std::runtime_error("-i and -o are required");
    return a;
}

mcpgpu::MIPrecision mi_precision(int method) {
    switch (method) {
        case 0: return mcpgpu::MIPrecision::FP32;
        case 2: return mcpgpu::MIPrecision::BF16X3;
        case 3: return mcpgpu::MIPrecision::BF16;
        case 4: return mcpgpu::MIPrecision::FP16;
        case 5: return mcpgpu::MIPrecision::FP16X3;
        default: throw std::runtime_error("unsupported MI method " + std::to_string(method) +
                                          " (0 = B-spline FP32, 2..5 = tensor-core forms)");
    }
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char** argv) {
    try {
        Args a = parse(argc, argv);
        Named in = read_matrix(a.in);
        double t0 = now_s();
        if (a.cmd == "convert") {
            write_matrix(a.out, in.m, in.rows, in.cols);
            return 0;
        }
        mcpgpu::Context ctx(0);
        if (a.cmd == "mi") {
            int method = a.methods.empty() ? 2 : a.methods[0];
            Matrix<float> mi;
            mcpgpu::compute_mi(ctx, in.m, a.bins, mi, mi_precision(method), a.order);
            std::printf("Computed,MI,,%.6f,sec\n", now_s() - t0);
            write_matrix(a.out, mi, in.rows, in.rows);
        } else if (a.cmd == "mcp") {
            int method = a.methods.empty() ? 1 : a.methods[0];
            if (method < 1 || method > 3) throw std::runtime_error("mcp -m must be 1 (MCP2), 2 (MCP3) or 3 (MCP4)");
            if (a.diagonal_set) mcpgpu::set_diagonal(in.m, a.diagonal);  // the mcp app resets only on request
            Matrix<float> ratio, maxmin;
            // the mcp app symmetrises MCP3 (apps/filter/mcp.cpp:463-476)
            mcpgpu::compute_mcp(ctx, in.m, method + 1, ratio, &maxmin, method == 2);
            std::printf("Compute MCP%d in %.6f sec\n", method + 1, now_s() - t0);
            if (!a.maxmin_out.empty()) write_matrix(a.maxmin_out, maxmin, in.rows, in.rows);
            write_matrix(a.out, ratio, in.rows, in.rows);
        } else if (a.cmd == "dpi") {
            mcpgpu::set_diagonal(in.m, a.diagonal);
            Matrix<float> out;
            int64_t removed = mcpgpu::dpi_filter(ctx, in.m, a.tol, out);
            std::printf("Mask removing %lld elements \n", (long long)removed);
            write_matrix(a.out, out, in.rows, in.rows);
        } else if (a.cmd == "mcpnet") {
            Matrix<float> mi;
            mcpgpu::compute_mi(ctx, in.m, a.bins, mi, mi_precision(a.mi_method), 3);
            std::printf("Computed,MI,,%.6f,sec\n", now_s() - t0);
            write_matrix(a.out + "_bs.mi" + (ends_with(a.in, ".bin") ? ".bin" : ".exp"), mi, in.rows, in.rows);
            mcpgpu::set_diagonal(mi, a.diagonal);
            std::vector<int> ms = a.methods.empty() ? std::vector<int>{1} : a.methods;
            for (int method : ms) {
                if (method < 1 || method > 3) throw std::runtime_error("mcpnet -m accepts 1, 2, 3");
                double t1 = now_s();
                Matrix<float> ratio;
                mcpgpu::compute_mcp(ctx, mi, method + 1, ratio);
                std::printf("Computed,MCP%d,,%.6f,sec\n", method + 1, now_s() - t1);
                write_matrix(a.out + "_bs.mcp" + std::to_string(method + 1) + (ends_with(a.in, ".bin") ? ".bin" : ".exp"),
                             ratio, in.rows, in.rows);
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
