// host_main.cpp -- command-line host for the TNF stages of MetaBAT2, a
// drop-in for the reference program's front half (cuda/Cuda2.cu:1251-1912):
// same flags, same input validation messages, same "# elapsed time (...)"
// lines (cuda/metrictime2.hpp), but every GPU stage runs through the C ABI of
// libmdet_tnf.so.  The reference continues into binning; this host runs
// its label propagation over the graph (sSCR = sTNF, the reference's path
// without a depth file, cuda/Cuda2.cu:1969-2061) and writes:
//   <out>.tnf_graph.tsv   name_i <TAB> name_j <TAB> sTNF   (i < j)
//   <out>.TNF.bin         n x 136 float64 rows c/sqrt(sum c^2), the TNF.bin
//                         layout of openmp/TNF.cpp
//   <out>.lp_bins.tsv     name <TAB> bin (the index of the contig whose label
//                         the bin carries), in input order
#include <charconv>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <memory>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

#include "mdet_tnf.h"

namespace {

struct Opts {
    std::string in, out, mode = "bf16";
    size_t min_contig = 2500, max_edges = 200, threads = 0;
    double maxP = 95, pTNF = 0, minS = 60;
    unsigned long long seed = 0;
    int ct = 32, device = 0;
    bool verbose = false, help = false, no_tnf_bin = false, no_bins = false;
};

using Clock = std::chrono::high_resolution_clock;

void timer_line(const char* label, Clock::time_point a) {
    std::chrono::duration<double> d = Clock::now() - a;
    std::cout << "# elapsed time (" << label << "): " << d.count() << "s" << std::endl;
}

void usage() {
    std::cerr << "\nMetaBAT 2 TNF stages on GB300 (mdet_tnf)\n\n"
                 "  -h [ --help ]             produce help message\n"
                 "  -i [ --inFile ] arg       Contigs in fasta file format [Mandatory]\n"
                 "  -o [ --outFile ] arg      Base file name for the TNF graph output [Mandatory]\n"
                 "  -m [ --minContig ] arg (=2500) Minimum size of a contig (should be >=1500)\n"
                 "  --maxP arg (=95)          Percentage of 'good' contigs considered for binning\n"
                 "  --minS arg (=60)          Minimum score of an edge (checked like the reference)\n"
                 "  --maxEdges arg (=200)     Maximum number of edges per node\n"
                 "  --pTNF arg (=0)           TNF probability cutoff for building TNF graph (0: auto)\n"
                 "  --seed arg (=0)           For exact reproducibility. (0: use random seed)\n"
                 "  -t [ --numThreads ] arg (=0) Number of host threads (accepted for compatibility)\n"
                 "  --ct arg (=32)            CUDA threads flag of the reference (multiple of 32; accepted)\n"
                 "  --mode arg (=bf16)        plain | bf16 : distance filter of the pairwise stage\n"
                 "  --device arg (=0)         CUDA device\n"
                 "  --noTNFbin                do not write <out>.TNF.bin\n"
                 "  --noBins                  skip label propagation and <out>.lp_bins.tsv\n"
                 "  -v [ --verbose ]          Verbose output\n";
}

bool parse(int ac, char** av, Opts& o) {
    for (int i = 1; i < ac; ++i) {
        std::string a = av[i];
        auto val = [&](std::string& dst) -> bool {
            size_t eq = a.find('=');
            if (eq != std::string::npos && a.rfind("--", 0) == 0) {
                dst = a.substr(eq + 1);
                return true;
            }
            if (a.size() > 2 && a[0] == '-' && a[1] != '-') {  // -iFILE
                dst = a.substr(2);
                return true;
            }
            if (i + 1 >= ac) return false;
            dst = av[++i];
            return true;
        };
        std::string key = a, v;
        size_t eq = a.find('=');
        if (eq != std::string::npos) key = a.substr(0, eq);
        if (key.size() > 2 && key[0] == '-' && key[1] != '-') key = key.substr(0, 2);
        if (key == "-h" || key == "--help") {
            o.help = true;
        } else if (key == "-v" || key == "--verbose") {
            o.verbose = true;
        } else if (key == "--noTNFbin") {
            o.no_tnf_bin = true;
        } else if (key == "--noBins") {
            o.no_bins = true;
        } else if (key == "-i" || key == "--inFile") {
            if (!val(o.in)) return false;
        } else if (key == "-o" || key == "--outFile") {
            if (!val(o.out)) return false;
        } else {
            if (!val(v)) return false;
            try {
                if (key == "-m" || key == "--minContig") o.min_contig = std::stoull(v);
                else if (key == "--maxP") o.maxP = std::stod(v);
                else if (key == "--minS") o.minS = std::stod(v);
                else if (key == "--maxEdges") o.max_edges = std::stoull(v);
                else if (key == "--pTNF") o.pTNF = std::stod(v);
                else if (key == "--seed") o.seed = std::stoull(v);
                else if (key == "-t" || key == "--numThreads") o.threads = std::stoull(v);
                else if (key == "--ct") o.ct = std::stoi(v);
                else if (key == "--mode") o.mode = v;
                else if (key == "--device") o.device = std::stoi(v);
                else {
                    std::cerr << "unrecognised option '" << a << "'" << std::endl;
                    return false;
                }
            } catch (...) {
                std::cerr << "the argument ('" << v << "') for option '" << key << "' is invalid" << std::endl;
                return false;
            }
        }
    }
    return true;
}

struct Fasta {
    char* mem = nullptr;  // page-locked (mdet_host_alloc)
    size_t size = 0;
    std::vector<std::string_view> names;
    std::vector<double> log_size;
    ~Fasta() { mdet_host_free(mem); }
};

// The file's bytes (the reference maps the whole file into pinned memory,
// cuda/Cuda2.cu:1459-1484); the record split runs on the GPU.
bool read_file(const std::string& path, Fasta& f) {
    std::ifstream is(path, std::ios::binary | std::ios::ate);
    if (!is) return false;
    const size_t fsize = (size_t)is.tellg();
    is.seekg(0);
    void* m = nullptr;
    if (mdet_host_alloc(fsize + 32, &m) != MDET_OK) return false;
    f.mem = (char*)m;
    f.size = fsize;
    is.read(f.mem, (std::streamsize)fsize);
    return (bool)is || fsize == 0;
}

int check(mdet_ctx* ctx, int rc, const char* what) {
    if (rc != MDET_OK) {
        std::cerr << "[Error!] " << what << ": " << mdet_last_error(ctx) << " (status " << rc << ")" << std::endl;
        exit(1);
    }
    return rc;
}

}  // namespace

int main(int ac, char** av) {
    Opts o;
    if (!parse(ac, av, o)) {
        usage();
        return 1;
    }
    if (o.help || o.in.empty() || o.out.empty()) {
        usage();
        if (!o.help) {
            if (o.in.empty()) std::cerr << "[Error!] There was no --inFile specified" << std::endl;
            if (o.out.empty()) std::cerr << "[Error!] There was no --outFile specified" << std::endl;
        }
        return o.help ? 0 : 1;
    }
    // validation as in cuda/Cuda2.cu:1311-1366
    if (o.seed == 0) o.seed = (unsigned long long)time(0);
    srand((unsigned)o.seed);
    if (o.maxP <= 0 || o.maxP >= 100) {
        std::cerr << "[Error!] maxP should be greater than 0 and less than 100" << std::endl;
        return 1;
    }
    if (o.minS <= 1 || o.minS >= 100) {
        std::cerr << "[Error!] minS should be greater than 1 and less than 100" << std::endl;
        return 1;
    }
    if (o.pTNF < 0 || o.pTNF >= 100) {
        std::cerr << "[Error!] pTNF should be >= 0 and < 100" << std::endl;
        return 1;
    }
    if (o.min_contig < 1500) {
        std::cerr << "[Error!] Contig length < 1500 is not allowed to be used for binning." << std::endl;
        return 1;
    }
    if (o.ct % 32 != 0) {
        std::cerr << "numThreads2 must be a multiple of 32" << std::endl;
        return 1;
    }
    int mode = o.mode == "plain" ? MDET_MODE_PLAIN : o.mode == "bf16" ? MDET_MODE_BF16 : -1;
    if (mode < 0) {
        std::cerr << "[Error!] --mode must be plain or bf16" << std::endl;
        return 1;
    }
    const double coverage = o.maxP / 100.;
    auto t_total = Clock::now();

    auto t_read = Clock::now();
    Fasta fa;
    if (!read_file(o.in, fa)) {
        std::cerr << "[Error!] can't open the sequence fasta file " << o.in << std::endl;
        return 1;
    }
    timer_line("read", t_read);
    auto t_abd = Clock::now();
    timer_line("ABD", t_abd);

    mdet_ctx* ctx = nullptr;
    if (mdet_ctx_create(o.device, &ctx) != MDET_OK) {
        std::cerr << "[Error!] no usable CUDA device " << o.device << std::endl;
        return 1;
    }
    // record split (reader rules of cuda/Cuda2.cu:1507-1544) and TNF counting
    // on the GPU, from one copy of the file
    auto t_tnf = Clock::now();
    uint64_t rcap = fa.size / 1000 + 16;
    // outputs sized for the largest possible count and left uninitialised
    // (only the first n rows are written, so only their pages are touched)
    std::unique_ptr<uint64_t[]> size, name_off;
    std::unique_ptr<uint32_t[]> name_len, counts_buf;
    std::unique_ptr<float[]> tnf_buf;
    mdet_fasta_stats fs;
    while (true) {
        size.reset(new uint64_t[rcap]);
        name_off.reset(new uint64_t[rcap]);
        name_len.reset(new uint32_t[rcap]);
        counts_buf.reset(new uint32_t[rcap * 136]);
        tnf_buf.reset(new float[rcap * 136]);
        int rc = mdet_tnf_count_fasta(ctx, fa.mem, fa.size, o.min_contig, rcap, nullptr, nullptr, size.get(),
                                      nullptr, name_off.get(), name_len.get(), counts_buf.get(), tnf_buf.get(),
                                      &fs);
        if (rc == MDET_ERR_CAPACITY && fs.n_large > rcap) {
            rcap = fs.n_large;
            continue;
        }
        check(ctx, rc, "TNF counting");
        break;
    }
    const uint64_t n = fs.n_large;
    for (uint64_t k = 0; k < n; ++k) {
        fa.names.emplace_back(fa.mem + name_off[k], name_len[k]);
        // log10(min(size, 500000)) on the host, as the reference computes it (cuda/Cuda2.cu:1535)
        fa.log_size.push_back(std::log10((double)std::min(size[k], (uint64_t)500000)));
    }
    {
        std::unordered_map<std::string_view, size_t> seen;
        for (size_t k = 0; k < fa.names.size(); ++k)
            if (!seen.emplace(fa.names[k], k).second) {
                std::cerr << "[Error!] Need to check whether there are duplicated sequence ids in the assembly file"
                          << std::endl;
                return 1;
            }
    }
    if (o.verbose) std::cout << "Number of large contigs >= " << o.min_contig << " are " << n << ". " << std::endl;
    const uint32_t* counts = counts_buf.get();
    const float* tnf = tnf_buf.get();
    timer_line("TNF_CAL", t_tnf);

    auto t_sample = Clock::now();
    double ptnf = o.pTNF;
    if (n >= 2 && ptnf < 1.)
        check(ctx, mdet_tnf_ptnf_search(ctx, tnf, fa.log_size.data(), n, coverage, mode, &ptnf), "pTNF search");
    else
        ptnf *= 10;
    if (o.verbose) printf("Finished Preparing TNF Graph Building [pTNF = %2.2f]\n", ptnf / 10.);
    timer_line("GRAPH_SAMPLE", t_sample);

    auto t_graph = Clock::now();
    uint64_t cap = n * o.max_edges + 1, ne = 0;
    // outputs left uninitialised: the call writes the first ne entries
    std::unique_ptr<uint64_t[]> from(new uint64_t[cap]), to(new uint64_t[cap]);
    std::unique_ptr<double[]> stnf(new double[cap]);
    mdet_graph_stats st;
    if (n >= 2)
        check(ctx, mdet_tnf_graph(ctx, tnf, fa.log_size.data(), n, ptnf / 1000., (uint32_t)o.max_edges, mode,
                                  from.get(), to.get(), stnf.get(), cap, &ne, &st),
              "TNF graph");
    timer_line("TNF_GRAPH", t_graph);
    if (ne == 0) std::cout << "No edges were formed by TNF." << std::endl;

    {
        FILE* g = fopen((o.out + ".tnf_graph.tsv").c_str(), "wb");
        if (!g) {
            std::cerr << "[Error!] can't open the output file: " << o.out << ".tnf_graph.tsv" << std::endl;
            return 1;
        }
        // shortest round-trip decimal of each sTNF (std::to_chars), written in
        // large blocks
        std::vector<char> blk(1 << 24);
        size_t used = 0;
        for (uint64_t e = 0; e < ne; ++e) {
            const std::string_view a = fa.names[from[e]], b = fa.names[to[e]];
            if (used + a.size() + b.size() + 40 > blk.size()) {
                if (a.size() + b.size() + 40 > blk.size()) blk.resize(2 * (a.size() + b.size() + 40));
                fwrite(blk.data(), 1, used, g);
                used = 0;
            }
            memcpy(blk.data() + used, a.data(), a.size());
            used += a.size();
            blk[used++] = '\t';
            memcpy(blk.data() + used, b.data(), b.size());
            used += b.size();
            blk[used++] = '\t';
            used = (size_t)(std::to_chars(blk.data() + used, blk.data() + blk.size(), stnf[e]).ptr - blk.data());
            blk[used++] = '\n';
        }
        fwrite(blk.data(), 1, used, g);
        if (fclose(g) != 0) {
            std::cerr << "[Error!] failed to write " << o.out << ".tnf_graph.tsv" << std::endl;
            return 1;
        }
    }
    if (!o.no_tnf_bin) {
        std::ofstream b(o.out + ".TNF.bin", std::ios::binary);
        std::vector<double> row(136);
        for (uint64_t r = 0; r < n; ++r) {
            double s = 0;
            for (int c = 0; c < 136; ++c) s += (double)counts[r * 136 + c] * (double)counts[r * 136 + c];
            s = std::sqrt(s);
            for (int c = 0; c < 136; ++c) row[c] = (double)counts[r * 136 + c] / s;
            b.write((const char*)row.data(), 136 * sizeof(double));
        }
    }
    if (!o.no_bins) {
        // binning by label propagation over the graph, sSCR = sTNF
        std::vector<uint64_t> mem(n);
        mdet_lp_stats lps{};
        if (n) check(ctx, mdet_label_propagation(ctx, from.get(), to.get(), stnf.get(), ne, n, o.maxP / 100.,
                                                 o.minS / 100., mem.data(), &lps),
                     "label propagation");
        if (o.verbose)
            printf("Label propagation: %llu runs, %llu sweeps over %llu edges of %llu contigs\n",
                   (unsigned long long)lps.calls, (unsigned long long)lps.sweeps,
                   (unsigned long long)lps.graph_edges, (unsigned long long)lps.connected);
        std::ofstream b(o.out + ".lp_bins.tsv");
        if (!b) {
            std::cerr << "[Error!] can't open the output file: " << o.out << ".lp_bins.tsv" << std::endl;
            return 1;
        }
        for (uint64_t r = 0; r < n; ++r) b << fa.names[r] << '\t' << mem[r] << '\n';
    }
    std::cout << ne << " edges" << std::endl;
    mdet_ctx_destroy(ctx);
    timer_line("total", t_total);
    return 0;
}
