// rtxrmq.cpp — benchmark driver with the reference's command line.
//
//   ./rtxrmq <n> <q> <lr> <alg> [options]
//
// Mirrors the reference driver (src/main.cu:71-287, arguments src/tools.h:92-259):
// generates the array and the inclusive queries on the host with the
// reference's generators, copies them to the device, runs one algorithm
// `reps` times, reports queries/s, optionally appends a CSV row, and checks
// the results against the brute-force GPU scan (--check, --trivialCheck,
// --randTrivialCheck; src/main.cu:194-283).  Checks here are bit-exact
// (the reference compares values with an absolute epsilon, src/tools.h:261).
//
// Algorithms of this driver:
//     0  [CPU] BASE            brute-force scan, OpenMP   (src/cpu_methods.h:18)
//   100  [CPU] BASE IDX        its argmin                 (src/cpu_methods.h:55)
//     2  [GPU] BASE            brute-force scan           (src/cuda_methods.cuh:72)
//   102  [GPU] BASE IDX        its argmin                 (src/cuda_methods.cuh:106)
//    22  [GPU] GB300 hierarchical min      (--variant cl|vl|auto)
//   122  [GPU] GB300 hierarchical argmin
// The reference's own ids 16 (CL) and 20 (VL) name its kernels; their GB300
// counterparts are 22 --variant cl and 22 --variant vl; its CL ablations 23, 24
// and 19 are 22 --variant cl-noshuffle, cl-tile and cl-atomic.
#include <getopt.h>
#include <omp.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rmq_gb300.h"
#include "../../include/rmq_gb300_gen.h"

namespace {

constexpr int ALG_CPU_BASE = 0;
constexpr int ALG_GPU_BASE = 2;
constexpr int ALG_GB300 = 22;
constexpr int ALG_CPU_BASE_IDX = 100;
constexpr int ALG_GPU_BASE_IDX = 102;
constexpr int ALG_GB300_IDX = 122;
constexpr uint32_t kTrivialQ = 1u << 10;      // TRIVCHECK_LOG_NUM_DIFFQ (src/main.cu:30)
constexpr uint32_t kRandTrivialQ = 1u << 15;  // RAND_TRIVCHECK_LOG_NUM_DIFFQ (src/main.cu:29)

struct Args {
    uint64_t n = 0;
    uint32_t q = 0;
    int lr = 0;
    int alg = -1;
    uint32_t log_bs = 15;
    int reps = 10;
    int dev = 0;
    int nt = 1;
    int seed = 0;
    int check = 0, trivial = 0, rand_trivial = 0;
    int save_time = 0, save_input = 0;
    std::string time_file, data_dir = ".";
    std::string variant = "auto";
    int rf_log = 0, lanes = 0, l2_persist = 0;
    double ties = 0.0;
    uint64_t nb = 0;               // --nb as given (0 = not given)
    int log_build_threshold = 0;   // accepted and recorded; no effect here
    int save_power = 0;            // accepted; power is not measured
    double hbm_peak = 0.0;         // GB/s for roofline_frac (0 = device theoretical)
};

const char* alg_name(int alg) {
    switch (alg) {
        case ALG_CPU_BASE: return "[CPU] BASE";
        case ALG_GPU_BASE: return "[GPU] BASE";
        case ALG_GB300: return "[GPU] GB300 HIERARCHICAL";
        case ALG_CPU_BASE_IDX: return "[CPU] BASE IDX";
        case ALG_GPU_BASE_IDX: return "[GPU] BASE IDX";
        case ALG_GB300_IDX: return "[GPU] GB300 HIERARCHICAL IDX";
        default: return "";
    }
}

void print_help() {
    std::fprintf(stderr,
                 "usage: ./rtxrmq <n> <q> <lr> <alg> [options]\n\n"
                 "  n    size of the fp32 array\n"
                 "  q    number of range-minimum queries\n"
                 "  lr   query length law (a length is between 1 and n):\n"
                 "         lr > 0  every query has length lr\n"
                 "         -1      length uniform over [1, n]\n"
                 "         -2, -3  lognormal lengths around n^0.6 / n^0.3 (sigma 0.3)\n"
                 "         -4, -5  lognormal lengths around n/2^8 / n/2^15 (sigma 0.3)\n"
                 "         -6      a random pick of -1, -2 or -3 per query\n"
                 "         -7      lognormal around 2^13 with sigma 1.0, clamped to [1, n]\n"
                 "         -8      thirds of: -1, lognormal(2^13, 1.0), lognormal(2^5, 0.7)\n"
                 "  alg  what answers the queries:\n"
                 "          0  CPU brute-force scan (OpenMP)\n"
                 "          2  GPU brute-force scan\n"
                 "         22  GPU hierarchy of block minima for GB300 (--variant cl|vl|auto)\n"
                 "         100, 102, 122: the same three returning the position of the minimum\n\n"
                 "options:\n"
                 "  --log_bs <k>            alg 22/122: scan threshold t = 2^k (default 2^15, at most n)\n"
                 "  --nb <blocks>           alg 22/122: t from a block count, t = 2^ceil(log2(n / blocks))\n"
                 "  --reps <r>              timed repetitions (default 10)\n"
                 "  --dev <id>              CUDA device (default 0)\n"
                 "  --nt <threads>          CPU threads of alg 0/100\n"
                 "  --seed <s>              generator seed (default: the clock)\n"
                 "  --check                 compare every result with the GPU brute-force scan, bit for bit\n"
                 "  --trivialCheck          only 2^10 distinct queries, repeated up to q, all compared\n"
                 "  --randTrivialCheck      compare a random sample of 2^15 results\n"
                 "  --save-time[=<file>]    append one CSV row of results (default ../results/data.csv)\n"
                 "  --save-input-data       keep generated inputs and expected results as raw files\n"
                 "  --data-dir <dir>        where those files go (default .)\n"
                 "  --log_build_threshold[=<k>]  accepted for command-line compatibility (no effect here)\n"
                 "  --save-power[=<file>]   accepted for command-line compatibility (power is not measured)\n"
                 "  --variant <name>        work distribution of alg 22/122: auto (default), vl, vl-short (vl\n"
                 "                          for short queries), cl, and the reference's ablations of cl:\n"
                 "                          cl-noshuffle (its alg 23), cl-tile (alg 24), cl-atomic (alg 19)\n"
                 "  --rf_log <3..5>         log2 of the per-level reduction factor (default: the variant's)\n"
                 "  --lanes <2|4|8|16|32>   CL lanes per query\n"
                 "  --l2_persist            put the coarse levels in an L2 persisting window\n"
                 "  --ties <frac>           set that fraction of the entries to the array's minimum\n"
                 "  --hbm_peak <GB/s>       peak for the CSV roofline_frac column (default: the device's\n"
                 "                          theoretical rate from its memory clock and bus width)\n");
}

// --variant names: the GB300 work distributions, and the reference's
// ablations of CL (its algs 23, 24 and 19) as work distributions of alg 22.
int variant_code(const std::string& v) {
    if (v == "cl") return RMQ_VARIANT_CL;
    if (v == "vl") return RMQ_VARIANT_VL;
    if (v == "vl-short") return RMQ_VARIANT_VL_SHORT;
    if (v == "cl-noshuffle") return RMQ_VARIANT_CL_NO_SHUFFLE;
    if (v == "cl-tile") return RMQ_VARIANT_CL_QUERY_PER_TILE;
    if (v == "cl-atomic") return RMQ_VARIANT_CL_ATOMIC;
    if (v == "auto") return RMQ_VARIANT_AUTO;
    return -1;
}

bool parse(int argc, char** argv, Args& a) {
    if (argc < 5) {
        print_help();
        return false;
    }
    a.n = std::strtoull(argv[1], nullptr, 10);
    a.q = uint32_t(std::strtoul(argv[2], nullptr, 10));
    a.lr = std::atoi(argv[3]);
    a.alg = std::atoi(argv[4]);
    if (!a.n || !a.q || !a.lr) {
        print_help();
        return false;
    }
    if (a.n > 0xFFFFFF00ull) {
        std::fprintf(stderr, "Error: n=%llu is above this driver's limit (uint32 queries)\n",
                     (unsigned long long)a.n);
        return false;
    }
    if (a.lr > 0 && uint64_t(a.lr) > a.n) {
        std::fprintf(stderr, "Error: lr=%i > n=%llu  (lr must be between '1' and 'n')\n", a.lr,
                     (unsigned long long)a.n);
        return false;
    }
    a.seed = int(std::time(nullptr));
    enum { O_BS = 1, O_REPS, O_DEV, O_NT, O_SEED, O_CHECK, O_TRIV, O_RTRIV, O_TIME, O_SAVE, O_DIR,
           O_VAR, O_RF, O_LANES, O_L2, O_TIES, O_NB, O_THRESH, O_POWER, O_PEAK };
    static option opts[] = {
        {"log_bs", required_argument, nullptr, O_BS},
        {"reps", required_argument, nullptr, O_REPS},
        {"dev", required_argument, nullptr, O_DEV},
        {"nt", required_argument, nullptr, O_NT},
        {"seed", required_argument, nullptr, O_SEED},
        {"check", no_argument, nullptr, O_CHECK},
        {"trivialCheck", no_argument, nullptr, O_TRIV},
        {"randTrivialCheck", no_argument, nullptr, O_RTRIV},
        {"save-time", optional_argument, nullptr, O_TIME},
        {"save-input-data", no_argument, nullptr, O_SAVE},
        {"data-dir", required_argument, nullptr, O_DIR},
        {"variant", required_argument, nullptr, O_VAR},
        {"rf_log", required_argument, nullptr, O_RF},
        {"lanes", required_argument, nullptr, O_LANES},
        {"l2_persist", no_argument, nullptr, O_L2},
        {"ties", required_argument, nullptr, O_TIES},
        {"nb", required_argument, nullptr, O_NB},
        {"log_build_threshold", optional_argument, nullptr, O_THRESH},
        {"save-power", optional_argument, nullptr, O_POWER},
        {"hbm_peak", required_argument, nullptr, O_PEAK},
        {nullptr, 0, nullptr, 0}};
    int opt, idx;
    optind = 5;
    while ((opt = getopt_long(argc, argv, "", opts, &idx)) != -1) {
        switch (opt) {
            case O_BS: {
                const uint32_t v = uint32_t(std::atoi(optarg));
                // clamp to floor(log2 n) as the reference does (src/tools.h:160)
                uint32_t fl = 0;
                while ((uint64_t(1) << (fl + 1)) <= a.n) ++fl;
                a.log_bs = (v < 64 && (uint64_t(1) << v) <= a.n) ? v : fl;
                break;
            }
            case O_REPS: a.reps = std::max(1, std::atoi(optarg)); break;
            case O_DEV: a.dev = std::atoi(optarg); break;
            case O_NT: a.nt = std::max(1, std::atoi(optarg)); break;
            case O_SEED: a.seed = std::atoi(optarg); break;
            case O_CHECK: a.check = 1; a.trivial = 0; a.rand_trivial = 0; break;
            case O_TRIV: a.trivial = 1; a.check = 0; a.rand_trivial = 0; break;
            case O_RTRIV: a.rand_trivial = 1; a.check = 0; a.trivial = 0; break;
            case O_TIME:
                a.save_time = 1;
                if (optarg) a.time_file = optarg;
                break;
            case O_SAVE: a.save_input = 1; break;
            case O_DIR: a.data_dir = optarg; break;
            case O_VAR: a.variant = optarg; break;
            case O_RF: a.rf_log = std::atoi(optarg); break;
            case O_LANES: a.lanes = std::atoi(optarg); break;
            case O_L2: a.l2_persist = 1; break;
            case O_TIES: a.ties = std::atof(optarg); break;
            case O_NB: {
                // as the reference (src/tools.h:168-175): nb = min(n, blocks),
                // t = 2^ceil(log2(n / nb)); a later --log_bs overrides it
                const long long v = std::atoll(optarg);
                if (v <= 0) {
                    std::fprintf(stderr, "Error: --nb needs a positive block count\n");
                    return false;
                }
                a.nb = std::min<uint64_t>(a.n, uint64_t(v));
                const uint64_t per = a.n / a.nb;
                uint32_t lg = 0;
                while ((uint64_t(1) << lg) < per) ++lg;
                a.log_bs = lg;
                break;
            }
            case O_THRESH:
                if (optarg) a.log_build_threshold = std::atoi(optarg);
                break;
            case O_POWER:
                a.save_power = 1;
                std::fprintf(stderr, "note: --save-power is accepted but power is not measured by this driver\n");
                break;
            case O_PEAK: a.hbm_peak = std::atof(optarg); break;
            default: print_help(); return false;
        }
    }
    if (variant_code(a.variant) < 0) {
        std::fprintf(stderr, "Error: unknown --variant %s\n", a.variant.c_str());
        return false;
    }
    // the default t = 2^15 is also clamped to log2(n)
    while (a.log_bs > 0 && (uint64_t(1) << a.log_bs) > a.n) --a.log_bs;
    if (a.time_file.empty()) a.time_file = "../results/data.csv";
    return true;
}

bool is_gpu_alg(int alg) {
    return alg == ALG_GPU_BASE || alg == ALG_GPU_BASE_IDX || alg == ALG_GB300 || alg == ALG_GB300_IDX;
}
bool is_idx_alg(int alg) { return alg >= 100; }

#define CK(x)                                                                                    \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) {                                                                 \
            std::fprintf(stderr, "%s:%d CUDA error: %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
            std::exit(EXIT_FAILURE);                                                             \
        }                                                                                        \
    } while (0)

#define RK(x)                                                                                    \
    do {                                                                                         \
        int s_ = (x);                                                                            \
        if (s_ != RMQ_OK) {                                                                      \
            std::fprintf(stderr, "%s:%d rmq error: %s\n", __FILE__, __LINE__, rmq_strerror(s_)); \
            std::exit(EXIT_FAILURE);                                                             \
        }                                                                                        \
    } while (0)

using Clock = std::chrono::high_resolution_clock;
double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

// The reference's brute-force CPU scan (src/cpu_methods.h:7-77): A[l] seeds
// the minimum, only a strictly smaller value replaces it.
void cpu_scan(const float* A, const uint32_t* Q, uint32_t q, float* out_min, uint32_t* out_idx, int nt) {
    omp_set_num_threads(nt);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < int64_t(q); ++i) {
        const uint32_t l = Q[2 * i], r = Q[2 * i + 1];
        float m = A[l];
        uint32_t mi = l;
        for (uint64_t j = l; j <= r; ++j) {
            if (A[j] < m) {
                m = A[j];
                mi = uint32_t(j);
            }
        }
        if (out_min) out_min[i] = m;
        if (out_idx) out_idx[i] = mi;
    }
}

std::string cache_name(const Args& a, const char* what, uint32_t q) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s/%s_n-%llu_q-%u_lr-%d_seed-%d_trivCheck-%d_randTrivCheck-%d.bin",
                  a.data_dir.c_str(), what, (unsigned long long)a.n, q, a.lr, a.seed, a.trivial,
                  a.rand_trivial);
    return buf;
}

bool load_raw(const std::string& f, void* dst, size_t bytes) {
    FILE* fp = std::fopen(f.c_str(), "rb");
    if (!fp) return false;
    const size_t got = std::fread(dst, 1, bytes, fp);
    std::fclose(fp);
    return got == bytes;
}

void save_raw(const std::string& f, const void* src, size_t bytes) {
    FILE* fp = std::fopen(f.c_str(), "wb");
    if (!fp) {
        std::fprintf(stderr, "warning: cannot write %s\n", f.c_str());
        return;
    }
    std::fwrite(src, 1, bytes, fp);
    std::fclose(fp);
}

// Algorithmic bytes of one query (the implementation-independent model the
// benchmark reports as roofline.achieved): the canonical descent with rf = 32
// reads, at level 0, the 32-byte sectors of [l, r] when the range has at most
// 64 entries, else those of [l, ceil32(l)) and [floor32(r + 1), r + 1).
uint64_t level0_sectors(uint64_t l, uint64_t r, uint64_t n) {
    const uint64_t e = r + 1, rf = 32;
    if (e - l <= 2 * rf || n <= 64) return (r >> 3) - (l >> 3) + 1;
    const uint64_t nl = (l + rf - 1) & ~(rf - 1), pr = e & ~(rf - 1);
    const uint64_t left = nl > l ? ((nl - 1) >> 3) - (l >> 3) + 1 : 0;
    const uint64_t right = e > pr ? (r >> 3) - (pr >> 3) + 1 : 0;
    return left + right;
}

// Sectors of levels >= 1 the same canonical descent (rf = 32, t = 64) reads:
// boundary pieces while it descends, then its final piece.
uint64_t coarse_sectors(uint64_t l, uint64_t r, uint64_t n) {
    const uint64_t rf = 32, t = 64;
    uint32_t top = 0;
    for (uint64_t size = n; top < 19 && size > t; size = (size + rf - 1) / rf) ++top;
    uint64_t lo = l, e = r + 1, total = 0;
    uint32_t k = 0;
    while (k < top && e - lo > 2 * rf) {
        const uint64_t nl = (lo + rf - 1) & ~(rf - 1), pr = e & ~(rf - 1);
        if (k > 0) {
            if (nl > lo) total += ((nl - 1) >> 3) - (lo >> 3) + 1;
            if (e > pr) total += ((e - 1) >> 3) - (pr >> 3) + 1;
        }
        lo = nl / rf;
        e = pr / rf;
        ++k;
    }
    if (k > 0 && e > lo) total += ((e - 1) >> 3) - (lo >> 3) + 1;
    return total;
}

struct Result {
    double total_ms = 0;     // host wall time of `reps` (launch + sync), reference style
    double event_ms = 0;     // device time of the median rep (CUDA events)
    float build_ms = 0;
    double out_mb = 0;
    std::vector<float> vmin;
    std::vector<uint32_t> vidx;
    rmq_info info{};
};

Result run_alg(const Args& a, const float* hA, const uint32_t* hQ, const float* dA, const uint32_t* dQ) {
    Result res;
    const uint32_t q = a.q;
    const bool idx = is_idx_alg(a.alg);
    if (idx) res.vidx.resize(q);
    else res.vmin.resize(q);
    if (!is_gpu_alg(a.alg)) {
        const auto t0 = Clock::now();
        for (int i = 0; i < a.reps; ++i)
            cpu_scan(hA, hQ, q, idx ? nullptr : res.vmin.data(), idx ? res.vidx.data() : nullptr, a.nt);
        res.total_ms = ms_since(t0);
        res.event_ms = res.total_ms / a.reps;
        return res;
    }
    float* dmin = nullptr;
    uint32_t* didx = nullptr;
    if (idx) CK(cudaMalloc(&didx, sizeof(uint32_t) * q));
    else CK(cudaMalloc(&dmin, sizeof(float) * q));
    rmq_handle* h = nullptr;
    if (a.alg == ALG_GB300 || a.alg == ALG_GB300_IDX) {
        rmq_config cfg;
        rmq_config_init(&cfg);
        cfg.variant = variant_code(a.variant);
        cfg.scan_threshold = uint64_t(1) << a.log_bs;
        cfg.rf_log = a.rf_log;
        cfg.lanes = a.lanes;
        cfg.l2_persist = a.l2_persist;
        cfg.with_index = idx ? 1 : 0;
        std::printf("Build GB300 hierarchy (%s, t=%llu)......", a.variant.c_str(),
                    (unsigned long long)cfg.scan_threshold);
        std::fflush(stdout);
        const int st = rmq_build(dA, a.n, &cfg, nullptr, &h);
        if (st != RMQ_OK) {
            std::fprintf(stderr, "\nError: rmq_build: %s\n", rmq_strerror(st));
            std::exit(EXIT_FAILURE);
        }
        RK(rmq_get_info(h, &res.info));
        res.build_ms = res.info.build_ms;
        res.out_mb = double(res.info.level_bytes) / 1e6;
        std::printf("done: %f ms (%u levels, rf=%u, %f MB)\n", res.build_ms, res.info.num_levels,
                    1u << res.info.rf_log, res.out_mb);
    }
    auto launch = [&]() {
        if (h == nullptr) {
            RK(rmq_scan_bruteforce(dA, a.n, dQ, q, dmin, didx, nullptr));
        } else if (idx) {
            RK(rmq_query_idx(h, dQ, q, didx, nullptr, nullptr));
        } else {
            RK(rmq_query(h, dQ, q, dmin, nullptr));
        }
    };
    launch();  // warm-up, not timed (the reference times cold launches; both are reported)
    CK(cudaDeviceSynchronize());
    std::vector<float> ev_ms;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const auto t0 = Clock::now();
    for (int i = 0; i < a.reps; ++i) {
        CK(cudaEventRecord(e0));
        launch();
        CK(cudaEventRecord(e1));
        CK(cudaDeviceSynchronize());
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        ev_ms.push_back(ms);
    }
    res.total_ms = ms_since(t0);
    std::sort(ev_ms.begin(), ev_ms.end());
    res.event_ms = ev_ms[ev_ms.size() / 2];
    if (idx) CK(cudaMemcpy(res.vidx.data(), didx, sizeof(uint32_t) * q, cudaMemcpyDeviceToHost));
    else CK(cudaMemcpy(res.vmin.data(), dmin, sizeof(float) * q, cudaMemcpyDeviceToHost));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    rmq_destroy(h);
    if (dmin) cudaFree(dmin);
    if (didx) cudaFree(didx);
    return res;
}

// Expected results from the brute-force GPU scan over `qs` (device copy made here).
void expected_on_gpu(const Args& a, const float* dA, const uint32_t* hq, uint32_t q,
                     std::vector<float>& emin, std::vector<uint32_t>& eidx) {
    uint32_t* dq = nullptr;
    float* dmin = nullptr;
    uint32_t* didx = nullptr;
    CK(cudaMalloc(&dq, sizeof(uint32_t) * 2 * q));
    CK(cudaMalloc(&dmin, sizeof(float) * q));
    CK(cudaMalloc(&didx, sizeof(uint32_t) * q));
    CK(cudaMemcpy(dq, hq, sizeof(uint32_t) * 2 * q, cudaMemcpyHostToDevice));
    RK(rmq_scan_bruteforce(dA, a.n, dq, q, dmin, didx, nullptr));
    emin.resize(q);
    eidx.resize(q);
    CK(cudaMemcpy(emin.data(), dmin, sizeof(float) * q, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(eidx.data(), didx, sizeof(uint32_t) * q, cudaMemcpyDeviceToHost));
    cudaFree(dq);
    cudaFree(dmin);
    cudaFree(didx);
}

int check(const Args& a, const float* hA, const uint32_t* hQ, const float* dA, const Result& r) {
    const bool idx = is_idx_alg(a.alg);
    // query positions to check and the queries themselves
    std::vector<uint32_t> pos;
    uint32_t nexp = a.q;
    if (a.trivial) nexp = std::min(a.q, kTrivialQ);
    if (a.rand_trivial) {
        pos.resize(std::min(a.q, kRandTrivialQ));
        pos.resize(rmq_gen_sample_indices(a.q, kRandTrivialQ, a.seed, pos.data()));
        nexp = uint32_t(pos.size());
    }
    std::vector<uint32_t> eq(2 * size_t(nexp));
    for (uint32_t i = 0; i < nexp; ++i) {
        const uint32_t src = a.rand_trivial ? pos[i] : i;
        eq[2 * i] = hQ[2 * size_t(src)];
        eq[2 * i + 1] = hQ[2 * size_t(src) + 1];
    }
    std::vector<float> emin;
    std::vector<uint32_t> eidx;
    const std::string fv = cache_name(a, "results_value", nexp), fi = cache_name(a, "results_index", nexp);
    emin.resize(nexp);
    eidx.resize(nexp);
    if (!(load_raw(fv, emin.data(), sizeof(float) * nexp) && load_raw(fi, eidx.data(), sizeof(uint32_t) * nexp))) {
        expected_on_gpu(a, dA, eq.data(), nexp, emin, eidx);
        if (a.save_input) {
            save_raw(fv, emin.data(), sizeof(float) * nexp);
            save_raw(fi, eidx.data(), sizeof(uint32_t) * nexp);
        }
    }
    uint64_t wrong = 0;
    const uint32_t total = a.rand_trivial ? nexp : a.q;
    for (uint32_t i = 0; i < total; ++i) {
        const uint32_t gi = a.rand_trivial ? pos[i] : i;           // position in the result
        const uint32_t ei = a.trivial ? (i & (kTrivialQ - 1)) : i;  // position in the expectation
        bool ok;
        if (idx) {
            ok = r.vidx[gi] == eidx[ei];
        } else {
            ok = std::memcmp(&r.vmin[gi], &emin[ei], sizeof(float)) == 0;
        }
        if (!ok) {
            if (wrong < 10) {
                if (idx)
                    std::printf("Error on %u-th query: got %u, expected %u  [%u,%u]\n", gi, r.vidx[gi], eidx[ei],
                                hQ[2 * size_t(gi)], hQ[2 * size_t(gi) + 1]);
                else
                    std::printf("Error on %u-th query: got %.10f, expected %.10f at idx %u  [%u,%u]\n", gi,
                                r.vmin[gi], emin[ei], eidx[ei], hQ[2 * size_t(gi)], hQ[2 * size_t(gi) + 1]);
            }
            ++wrong;
        }
    }
    (void)hA;
    if (wrong) std::printf("%.2f%% wrong.\n", 100.0 * double(wrong) / double(total));
    return wrong == 0 ? 1 : 0;
}

void write_csv(const Args& a, const Result& r, const uint32_t* hQ, int check_code) {
    if (!a.save_time) return;
    const bool hier = a.alg == ALG_GB300 || a.alg == ALG_GB300_IDX;
    FILE* probe = std::fopen(a.time_file.c_str(), "r");
    const bool exists = probe != nullptr;
    if (probe) std::fclose(probe);
    FILE* fp = std::fopen(a.time_file.c_str(), "a");
    if (!fp) {
        std::fprintf(stderr, "warning: cannot open %s\n", a.time_file.c_str());
        return;
    }
    // Column schema of create_XXX_header / create_header (src/tools.h:508-524);
    // this driver's columns follow checkResult.
    const char* extra = "variant,rf_log,lanes,event_qps,hbm_GBps,l2_GBps,roofline_frac,p50_us,p99_us,mode,"
                        "hbm_peak_GBps\n";
    if (!exists) {
        if (hier)
            std::fprintf(fp, "dev,alg,nt,reps,n,bs,nb,q,lr,GPU_BSIZE,CG_GROUP_SIZE,CG_MEM_ALIGNMENT,timestamp,"
                             "scan_threshold,XXX_CG_SIZE_LOG,XXX_CG_AMOUNT_LOG,t,q/s,ns/q,construction,outbuffer,"
                             "tempbuffer,freeGPUMemCorrect,freeGPUMem,checkResult,%s", extra);
        else
            std::fprintf(fp, "dev,alg,nt,reps,n,bs,nb,q,lr,GPU_BSIZE,CG_GROUP_SIZE,CG_MEM_ALIGNMENT,timestamp,t,"
                             "q/s,ns/q,construction,outbuffer,tempbuffer,freeGPUMemCorrect,freeGPUMem,checkResult,%s",
                         extra);
    }
    char device[300] = "CPU";
    if (is_gpu_alg(a.alg)) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, a.dev) == cudaSuccess) std::snprintf(device, sizeof(device), "%s", p.name);
    } else {
        char host[128] = "";
        gethostname(host, sizeof(host) - 1);
        std::snprintf(device, sizeof(device), "CPU %s (%d threads)", host, a.nt);
    }
    char ts[32];
    const std::time_t now = std::time(nullptr);
    std::strftime(ts, sizeof(ts), "%Y-%m-%dT%H:%M:%SZ", std::localtime(&now));
    size_t free_b = 0, total_b = 0;
    const int mem_ok = is_gpu_alg(a.alg) && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess ? 1 : 0;
    const double t_it = r.total_ms / a.reps;
    const int gpu_bsize = is_gpu_alg(a.alg) ? 256 : 0;
    // bs and nb as the reference writes them: 1 and 0 for its hierarchy rows
    // (src/tools.h:385-392), and for every algorithm whose block size it
    // resets (src/tools.h:221-235), which covers all of this driver's.
    const bool vl = r.info.variant == RMQ_VARIANT_VL || r.info.variant == RMQ_VARIANT_VL_SHORT;
    int size_log = 0;
    while (size_log < 6 && (1 << size_log) < r.info.lanes) ++size_log;
    // XXX_CG_SIZE_LOG: log2 of the lanes per query, 0 for VL (src/tools.h:403);
    // XXX_CG_AMOUNT_LOG: log2 of the entries per lane and level step, rf / lanes
    // (CL) or rf / 4 (VL, whose build uses 4-lane tiles, src/xxx.h:1002).
    const int cg_size_log = vl ? 0 : size_log;
    const int cg_amount_log = int(r.info.rf_log) - (vl ? 2 : size_log);
    if (hier)
        std::fprintf(fp, "%s,%s,%d,%d,%llu,1,0,%u,%d,%d,0,0,%s,%llu,%d,%d,", device, alg_name(a.alg), a.nt, a.reps,
                     (unsigned long long)a.n, a.q, a.lr, gpu_bsize, ts, (unsigned long long)(uint64_t(1) << a.log_bs),
                     cg_size_log, cg_amount_log);
    else
        std::fprintf(fp, "%s,%s,%d,%d,%llu,1,0,%u,%d,%d,0,0,%s,", device, alg_name(a.alg), a.nt, a.reps,
                     (unsigned long long)a.n, a.q, a.lr, gpu_bsize, ts);
    // outbuffer: the level buffer of block minima (MB), as the reference
    // (src/xxx.h:269); tempbuffer: the stored argmin positions beside it.
    const bool idx = is_idx_alg(a.alg);
    const double lvl_mb = hier ? double(r.info.level_bytes) / 1e6 : 0.0;
    const double out_mb = idx ? lvl_mb / 2 : lvl_mb, tmp_mb = idx ? lvl_mb / 2 : 0.0;
    std::fprintf(fp, "%f,%f,%f,%f,%f,%f,%d,%f,%d,", r.total_ms / 1000.0, double(a.q) / (t_it / 1000.0),
                 t_it * 1e6 / a.q, double(r.build_ms), out_mb, tmp_mb, mem_ok, double(free_b) / 1048576.0,
                 check_code);
    std::fprintf(fp, "%s,%d,%d,%f,", hier ? a.variant.c_str() : "", hier ? int(r.info.rf_log) : 0,
                 hier ? r.info.lanes : 0, double(a.q) / (r.event_ms / 1000.0));
    if (hier && r.event_ms > 0) {
        uint64_t b0 = 0, b1 = 0;
        for (uint64_t i = 0; i < a.q; ++i) {
            b0 += level0_sectors(hQ[2 * i], hQ[2 * i + 1], a.n);
            b1 += coarse_sectors(hQ[2 * i], hQ[2 * i + 1], a.n);
        }
        const double hbm_bytes = double(a.q) * (8 + 4) + 32.0 * double(b0);
        const double hbm = hbm_bytes / (r.event_ms / 1e3) / 1e9, l2 = 32.0 * double(b1) / (r.event_ms / 1e3) / 1e9;
        double peak = a.hbm_peak;
        if (!(peak > 0)) {
            int clk_khz = 0, bus_bits = 0;
            if (cudaDeviceGetAttribute(&clk_khz, cudaDevAttrMemoryClockRate, a.dev) == cudaSuccess &&
                cudaDeviceGetAttribute(&bus_bits, cudaDevAttrGlobalMemoryBusWidth, a.dev) == cudaSuccess)
                peak = 2.0 * double(clk_khz) * 1e3 * (bus_bits / 8.0) / 1e9;
            cudaGetLastError();
        }
        std::fprintf(fp, "%f,%f,", hbm, l2);
        if (peak > 0) std::fprintf(fp, "%f,,,plain,%f\n", hbm / peak, peak);
        else std::fprintf(fp, ",,,plain,\n");
    } else {
        std::fprintf(fp, ",,,,,%s,\n", is_gpu_alg(a.alg) ? "plain" : "cpu");
    }
    std::fclose(fp);
}

}  // namespace

int main(int argc, char** argv) {
    std::printf("----------------------------------\n");
    std::printf("   RMQ on GB300 (rtxrmq driver)   \n");
    std::printf("----------------------------------\n");
    Args a;
    if (!parse(argc, argv, a)) return EXIT_FAILURE;
    if (a.alg == 16 || a.alg == 20 || a.alg == 17 || a.alg == 18 || a.alg == 19 || a.alg == 21 ||
        a.alg == 23 || a.alg == 24) {
        std::fprintf(stderr, "Error: alg %d is one of the reference's own kernels; this driver runs "
                             "alg 22 --variant cl (CL, alg 16), vl (VL, alg 20), cl-noshuffle (alg 23), "
                             "cl-tile (alg 24) or cl-atomic (alg 19)\n", a.alg);
        return EXIT_FAILURE;
    }
    if (std::string(alg_name(a.alg)).empty()) {
        std::fprintf(stderr, "Error: alg %d is not available in this driver\n", a.alg);
        print_help();
        return EXIT_FAILURE;
    }
    std::printf("Params:\n   reps = %d\n   seed = %d\n   dev  = %d\n   n    = %llu (~%f GB, float)\n"
                "   t    = %llu\n   q    = %u (~%f GB, int2)\n   lr   = %d\n   nt   = %d CPU threads\n"
                "   alg  = %d (%s)\n\n",
                a.reps, a.seed, a.dev, (unsigned long long)a.n, 4.0 * a.n / 1e9,
                (unsigned long long)(uint64_t(1) << a.log_bs), a.q, 8.0 * a.q / 1e9, a.lr, a.nt, a.alg,
                alg_name(a.alg));
    const bool need_gpu = is_gpu_alg(a.alg) || a.check || a.trivial || a.rand_trivial;
    if (need_gpu) CK(cudaSetDevice(a.dev));

    auto t0 = Clock::now();
    std::printf("Generating n=%-10llu values............", (unsigned long long)a.n);
    std::fflush(stdout);
    std::vector<float> hA(a.n);
    const std::string fa = a.data_dir + "/array_n-" + std::to_string(a.n) + "_seed-" + std::to_string(a.seed) +
                           (a.ties > 0 ? "_ties-" + std::to_string(a.ties) : std::string()) + ".bin";
    if (!load_raw(fa, hA.data(), sizeof(float) * a.n)) {
        rmq_gen_array(a.n, a.seed, hA.data());
        if (a.ties > 0) rmq_gen_plant_min_ties(hA.data(), a.n, a.ties, a.seed);
        if (a.save_input) save_raw(fa, hA.data(), sizeof(float) * a.n);
    }
    std::printf("done: %f secs\n", ms_since(t0) / 1000);
    t0 = Clock::now();
    std::printf("Generating q=%-10u queries...........", a.q);
    std::fflush(stdout);
    std::vector<uint32_t> hQ(2 * size_t(a.q));
    const std::string fq = cache_name(a, "queries", a.q);
    if (!load_raw(fq, hQ.data(), sizeof(uint32_t) * 2 * a.q)) {
        if (rmq_gen_queries(a.q, a.lr, a.n, a.seed, a.trivial, hQ.data()) != 0) {
            std::fprintf(stderr, "\nError: unknown length law lr=%d\n", a.lr);
            return EXIT_FAILURE;
        }
        if (a.save_input) save_raw(fq, hQ.data(), sizeof(uint32_t) * 2 * a.q);
    }
    std::printf("done: %f secs\n", ms_since(t0) / 1000);

    float* dA = nullptr;
    uint32_t* dQ = nullptr;
    if (need_gpu) {
        CK(cudaMalloc(&dA, sizeof(float) * a.n));
        CK(cudaMemcpy(dA, hA.data(), sizeof(float) * a.n, cudaMemcpyHostToDevice));
        CK(cudaMalloc(&dQ, sizeof(uint32_t) * 2 * size_t(a.q)));
        CK(cudaMemcpy(dQ, hQ.data(), sizeof(uint32_t) * 2 * size_t(a.q), cudaMemcpyHostToDevice));
    }

    std::printf("Computing RMQs (%s, r=%d).....", alg_name(a.alg), a.reps);
    std::fflush(stdout);
    Result r = run_alg(a, hA.data(), hQ.data(), dA, dQ);
    const double avg_s = r.total_ms / (1000.0 * a.reps);
    std::printf("done: %f secs (avg %f secs) [%.2f RMQs/sec]  device median %f ms [%.2f RMQs/sec]\n",
                r.total_ms / 1000, avg_s, double(a.q) / avg_s, r.event_ms, double(a.q) / (r.event_ms / 1000));

    int check_code = -1;
    if (a.check || a.trivial || a.rand_trivial) {
        std::printf("\nCHECKING RESULT%s:\nChecking result...........................",
                    a.trivial ? " (trivial)" : a.rand_trivial ? " (random sample)" : "");
        const int pass = check(a, hA.data(), hQ.data(), dA, r);
        std::printf("%s\n", pass ? "pass" : "failed");
        check_code = pass + (a.trivial ? 2 : 0) + (a.rand_trivial ? 4 : 0);
    }
    write_csv(a, r, hQ.data(), check_code);
    if (dA) cudaFree(dA);
    if (dQ) cudaFree(dQ);
    std::printf("Benchmark Finished\n");
    return check_code == 0 || check_code == 2 || check_code == 4 ? 2 : 0;
}
