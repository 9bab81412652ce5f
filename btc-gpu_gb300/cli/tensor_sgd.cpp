// tensor_sgd -- drop-in command line of the GB300 CP-SGD path.
//
// Same arguments, input files, output files and stdout lines as the
// reference binary (main.cpp:101-316, tensor_SGD.cu:55-90,
// sgd_Kernel.cu:968-1361), driven through the C ABI in btc_gpu.h:
//
//   tensor_sgd <dataset> <I> <J> <K> [data_dir] [coord_base] [output_dir]
//              [--epochs N] [--rank|--r N] [--lr X] [--reg X]
//              [--block|--block-s|--block_s N] [--thread-size|--thread_size N]
//              [--parallel-sequence-size|--parallel_sequence_size N]
//              [--gpus|--gpu-count|--gpu_count N]
//
// Options added to the reference's command line (none collide with its own):
//   --precision f32|f64|bf16   factor storage / math (default f32)
//   --mode hogwild|deterministic|staged|lockfree   kernel schedule (default hogwild)
//   --seed N                   seeded U(init-lo, init-hi) factor init; without it
//                              the init is drawn from std::random_device like
//                              the reference (tensor_SGD.cu:43-53)
//   --init-lo X --init-hi X    init range (default 0.02, 0.1 as the reference)
//   --init-file FILE           initial factors as raw doubles A[I*r], B[J*r], C[K*r]
//   --dump-factors DIR         write A.txt, B.txt, C.txt (rows of %.17g)
//   --device N                 CUDA device ordinal
//   --bin-cache DIR            keep parsed train/test files as binary caches
//                              in DIR (<file name>.btcbin) and read them
//                              instead of the text while they match
#include <sys/stat.h>

#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "btc_gpu.h"

using std::cerr;
using std::cout;
using std::endl;
using std::string;

namespace {

btc_config cfg;
string dataset_name = "tensor";
string output_root = "output";
string precision = "f32", mode_name = "hogwild", dump_dir, init_file, bin_cache_dir;
bool have_seed = false;
unsigned long long seed = 0;
double init_lo = 0.02, init_hi = 0.1;

string join_path(const string& dir, const string& name)
{
    if (dir.empty())
        return name;
    char last = dir[dir.size() - 1];
    if (last == '/' || last == '\\')
        return dir + name;
    return dir + "/" + name;
}

// mkdir -p without a shell: every prefix of `path` that ends at a '/' is
// created with mkdir(2) (existing directories are fine), so no character of
// the path is ever interpreted as a command.
bool make_dirs(const string& path)
{
    if (path.empty())
        return true;
    for (size_t i = 1; i <= path.size(); i++) {
        if (i < path.size() && path[i] != '/')
            continue;
        const string part = path.substr(0, i);
        if (part.empty() || part == "/")
            continue;
        if (mkdir(part.c_str(), 0777) != 0 && errno != EEXIST)
            return false;
    }
    struct stat st;
    return stat(path.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

void print_usage(const char* program)
{
    cerr << "Usage: " << program << " <dataset> <I> <J> <K> [data_dir] [coord_base] [output_dir] [options]" << endl;
    cerr << "Example: " << program
         << " delicious-3d 532924 17262471 2480308 /fan/data 1 /fan/output --epochs 1000 --rank 4 --lr 0.001 "
            "--reg 0.05 --block 1024 --parallel-sequence-size 8 --gpus 4"
         << endl;
    cerr << "Reads <dataset>.train and <dataset>.test from data_dir." << endl;
    cerr << "Options:" << endl;
    cerr << "  --epochs N                    Training epochs. Default: " << cfg.epochs << endl;
    cerr << "  --rank N, --r N               Factor rank r. Default: " << cfg.rank << endl;
    cerr << "  --lr VALUE                    Learning rate. Default: " << cfg.lr << endl;
    cerr << "  --reg VALUE                   Regularization. Default: " << cfg.reg << endl;
    cerr << "  --block N, --block-s N, --block_s N" << endl;
    cerr << "                                Block size. Default: " << cfg.block_s << endl;
    cerr << "  --thread-size N, --thread_size N" << endl;
    cerr << "                                CUDA threads per block. Default: " << cfg.thread_size << endl;
    cerr << "  --parallel-sequence-size N, --parallel_sequence_size N" << endl;
    cerr << "                                Fixed blocks per parallel sequence; 0 means auto. Default: "
         << cfg.parallel_sequence_size << endl;
    cerr << "  --gpus N, --gpu-count N, --gpu_count N" << endl;
    cerr << "                                GPUs to use; 0 means all visible GPUs. Default: "
         << cfg.requested_gpu_count << endl;
    cerr << "  --precision f32|f64|bf16      Factor precision. Default: f32" << endl;
    cerr << "  --mode hogwild|deterministic|staged|lockfree   Kernel schedule. Default: hogwild" << endl;
    cerr << "  --seed N                      Seeded factor init (default: random_device)" << endl;
    cerr << "  --init-lo X, --init-hi X      Factor init range. Default: 0.02 0.1" << endl;
    cerr << "  --init-file FILE              Initial factors (raw doubles A, B, C)" << endl;
    cerr << "  --dump-factors DIR            Write the final factors as text" << endl;
    cerr << "  --device N                    CUDA device. Default: 0" << endl;
    cerr << "  --bin-cache DIR               Binary caches of the parsed input files" << endl;
}

bool read_option_value(const string& arg, int& index, int argc, char** argv, string& option, string& value)
{
    size_t eq = arg.find('=');
    if (eq != string::npos) {
        option = arg.substr(0, eq);
        value = arg.substr(eq + 1);
        return true;
    }
    option = arg;
    if (index + 1 >= argc) {
        cerr << "Missing value for option " << option << endl;
        return false;
    }
    index++;
    value = argv[index];
    return true;
}

bool apply_option(const string& o, const string& v)
{
    if (o == "--epochs")
        cfg.epochs = atoi(v.c_str());
    else if (o == "--rank" || o == "--r")
        cfg.rank = atoi(v.c_str());
    else if (o == "--lr")
        cfg.lr = atof(v.c_str());
    else if (o == "--reg")
        cfg.reg = atof(v.c_str());
    else if (o == "--block" || o == "--block-s" || o == "--block_s")
        cfg.block_s = atoi(v.c_str());
    else if (o == "--thread-size" || o == "--thread_size")
        cfg.thread_size = atoi(v.c_str());
    else if (o == "--parallel-sequence-size" || o == "--parallel_sequence_size")
        cfg.parallel_sequence_size = atoi(v.c_str());
    else if (o == "--gpus" || o == "--gpu-count" || o == "--gpu_count")
        cfg.requested_gpu_count = atoi(v.c_str());
    else if (o == "--precision")
        precision = v;
    else if (o == "--mode")
        mode_name = v;
    else if (o == "--seed") {
        have_seed = true;
        seed = strtoull(v.c_str(), nullptr, 10);
    } else if (o == "--init-lo")
        init_lo = atof(v.c_str());
    else if (o == "--init-hi")
        init_hi = atof(v.c_str());
    else if (o == "--dump-factors")
        dump_dir = v;
    else if (o == "--init-file")
        init_file = v;
    else if (o == "--device")
        cfg.device = atoi(v.c_str());
    else if (o == "--bin-cache")
        bin_cache_dir = v;
    else {
        cerr << "Unknown option: " << o << endl;
        return false;
    }
    return true;
}

bool validate_runtime_config()
{
    if (cfg.epochs <= 0) {
        cerr << "epochs must be positive." << endl;
        return false;
    }
    if (cfg.rank <= 0 || cfg.rank > 100) {
        cerr << "rank r must be in [1, 100]. The current CUDA kernel uses fixed local arrays of length 100." << endl;
        return false;
    }
    if (cfg.lr <= 0) {
        cerr << "lr must be positive." << endl;
        return false;
    }
    if (cfg.reg < 0) {
        cerr << "reg must be non-negative." << endl;
        return false;
    }
    if (cfg.block_s <= 0) {
        cerr << "block must be positive." << endl;
        return false;
    }
    if (cfg.thread_size <= 0 || cfg.thread_size > 1024) {
        cerr << "thread-size must be in [1, 1024]." << endl;
        return false;
    }
    if (cfg.parallel_sequence_size < 0) {
        cerr << "parallel-sequence-size must be >= 0." << endl;
        return false;
    }
    if (cfg.requested_gpu_count < 0) {
        cerr << "gpus must be >= 0. Use 0 for all visible GPUs." << endl;
        return false;
    }
    if (precision == "f32")
        cfg.dtype = BTC_DTYPE_F32;
    else if (precision == "f64")
        cfg.dtype = BTC_DTYPE_F64;
    else if (precision == "bf16")
        cfg.dtype = BTC_DTYPE_BF16;
    else {
        cerr << "precision must be f32, f64 or bf16." << endl;
        return false;
    }
    if (mode_name == "hogwild")
        cfg.mode = BTC_MODE_HOGWILD;
    else if (mode_name == "deterministic")
        cfg.mode = BTC_MODE_DETERMINISTIC;
    else if (mode_name == "staged")
        cfg.mode = BTC_MODE_STAGED;
    else if (mode_name == "lockfree")
        cfg.mode = BTC_MODE_LOCKFREE;
    else {
        cerr << "mode must be hogwild, deterministic, staged or lockfree." << endl;
        return false;
    }
    if (!(init_hi >= init_lo)) {
        cerr << "init-hi must be >= init-lo." << endl;
        return false;
    }
    return true;
}

void print_runtime_config()
{
    cout << "Runtime config:"
         << " epochs=" << cfg.epochs << " r=" << cfg.rank << " lr=" << cfg.lr << " reg=" << cfg.reg
         << " block_s=" << cfg.block_s << " thread_size=" << cfg.thread_size
         << " parallel_sequence_size=" << cfg.parallel_sequence_size
         << " requested_gpus=" << cfg.requested_gpu_count << endl;
}

bool file_exists(const string& p)
{
    std::ifstream f(p.c_str());
    return f.is_open();
}

struct Entries {
    int32_t* xyz = nullptr;
    double* val = nullptr;
    int64_t n = 0;
    ~Entries()
    {
        btc_free(xyz);
        btc_free(val);
    }
};

// read_entries (main.cpp:65-99); exits like the reference on failure
void read_entries(const std::vector<string>& cands, const string& label, int coord_base, Entries& out)
{
    string opened;
    for (const auto& c : cands)
        if (file_exists(c)) {
            opened = c;
            break;
        }
    if (opened.empty()) {
        cerr << "Failed to open " << label << " file. Tried:" << endl;
        for (const auto& c : cands)
            cerr << "  " << c << endl;
        exit(1);
    }
    int64_t line = 0;
    btc_status st;
    if (bin_cache_dir.empty()) {
        st = btc_read_entries(opened.c_str(), coord_base, cfg.I, cfg.J, cfg.K, &out.xyz, &out.val, &out.n, &line);
    } else {
        const size_t slash = opened.find_last_of('/');
        const string cache = join_path(bin_cache_dir, opened.substr(slash == string::npos ? 0 : slash + 1) + ".btcbin");
        int32_t from_cache = 0;
        st = btc_read_entries_cached(opened.c_str(), cache.c_str(), coord_base, cfg.I, cfg.J, cfg.K, &out.xyz,
                                     &out.val, &out.n, &line, &from_cache);
        if (st == BTC_OK)
            cerr << (from_cache ? "Read " : "Parsed the text; refreshed (where writable) ") << label
                 << " binary cache " << cache << endl;
    }
    if (st == BTC_ERR_RANGE) {
        std::ifstream f(opened.c_str());
        string s;
        for (int64_t i = 0; i < line && std::getline(f, s); i++) {
        }
        long long x = 0, y = 0, z = 0;
        std::stringstream ss(s);
        ss >> x >> y >> z;
        cerr << "Invalid " << label << " coordinate at " << opened << ":" << line << " -> (" << x - coord_base
             << "," << y - coord_base << "," << z - coord_base << ") after base conversion" << endl;
        exit(1);
    }
    if (st != BTC_OK) {
        cerr << "Failed to read " << label << " file " << opened << ": " << btc_status_string(st) << endl;
        exit(1);
    }
    cout << "Loaded " << out.n << " " << label << " entries from " << opened << endl;
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::system_clock::now().time_since_epoch()).count();
}

void fail(btc_status st, const char* what)
{
    cerr << what << " failed: " << btc_status_string(st) << endl;
    exit(1);
}

void write_factor(const string& path, const std::vector<double>& m, int64_t rows, int r)
{
    FILE* f = fopen(path.c_str(), "w");
    if (!f) {
        cerr << "Failed to open " << path << endl;
        return;
    }
    for (int64_t i = 0; i < rows; i++) {
        for (int q = 0; q < r; q++)
            fprintf(f, q ? " %.17g" : "%.17g", m[(size_t)i * r + q]);
        fprintf(f, "\n");
    }
    fclose(f);
}

}  // namespace

int main(int argc, char** argv)
{
    btc_config_default(&cfg);
    if (argc > 1 && (string(argv[1]) == "--help" || string(argv[1]) == "-h")) {
        print_usage(argv[0]);
        return 0;
    }
    if (argc < 5) {
        print_usage(argv[0]);
        return 1;
    }
    dataset_name = argv[1];
    cfg.I = atoi(argv[2]);
    cfg.J = atoi(argv[3]);
    cfg.K = atoi(argv[4]);
    std::vector<string> positional;
    for (int index = 5; index < argc; index++) {
        string arg = argv[index];
        if (arg == "--help" || arg == "-h") {
            print_usage(argv[0]);
            return 0;
        }
        if (arg.size() > 2 && arg.substr(0, 2) == "--") {
            string option, value;
            if (!read_option_value(arg, index, argc, argv, option, value) || !apply_option(option, value)) {
                print_usage(argv[0]);
                return 1;
            }
        } else {
            positional.push_back(arg);
        }
    }
    string data_dir = positional.size() > 0 ? positional[0] : "/fan/data";
    int coord_base = positional.size() > 1 ? atoi(positional[1].c_str()) : 1;
    output_root = positional.size() > 2 ? positional[2] : "output";
    if (cfg.I <= 0 || cfg.J <= 0 || cfg.K <= 0) {
        cerr << "I, J, and K must be positive." << endl;
        return 1;
    }
    if (coord_base != 0 && coord_base != 1) {
        cerr << "coord_base must be 0 or 1." << endl;
        return 1;
    }
    if (positional.size() > 3) {
        cerr << "Too many positional arguments." << endl;
        print_usage(argv[0]);
        return 1;
    }
    if (!validate_runtime_config())
        return 1;

    int32_t ndev = 0;
    btc_status st = btc_device_count(&ndev);
    if (st != BTC_OK && st != BTC_ERR_NO_DEVICE) {
        cerr << "cudaGetDeviceCount failed: " << btc_status_string(st) << endl;
        return 1;
    }
    cout << "CUDA visible GPU count=" << ndev << endl;
    if (ndev <= 0) {
        cerr << "No visible CUDA GPU devices." << endl;
        return 1;
    }
    print_runtime_config();

    Entries train, test;
    read_entries({join_path(data_dir, dataset_name + ".train"), join_path(data_dir, dataset_name + "_tr.tns"),
                  join_path(data_dir, dataset_name + ".tr.tns")},
                 "train", coord_base, train);
    read_entries({join_path(data_dir, dataset_name + ".test"), join_path(data_dir, dataset_name + "_te.tns"),
                  join_path(data_dir, dataset_name + ".te.tns")},
                 "test", coord_base, test);
    if (train.n == 0) {
        cerr << "Train file has no entries." << endl;
        return 1;
    }
    if (train.n > 1) {
        btc_shuffle_entries(train.xyz, train.val, train.n, 42);
        cout << "Shuffled train entries with seed=42 before block construction." << endl;
    }
    long long total = (long long)train.n + (long long)test.n;
    double train_rate = total > 0 ? (double)train.n / (double)total : 0.0;
    cout << "Train rate=" << train_rate << " test rate=" << (1.0 - train_rate) << endl;

    // tensor_SGD (tensor_SGD.cu:55-90)
    cout << "dataset=" << dataset_name << " dims=" << cfg.I << "x" << cfg.J << "x" << cfg.K
         << " train_nnz=" << train.n << " test_nnz=" << test.n << endl;
    const int r = cfg.rank;
    const int64_t rows[3] = {cfg.I, cfg.J, cfg.K};
    std::vector<double> F[3];
    {
        std::random_device rd;
        std::mt19937_64 gen(have_seed ? seed : ((unsigned long long)rd() << 32 | rd()));
        std::uniform_real_distribution<double> dist(init_lo, init_hi);
        for (int m = 0; m < 3; m++) {
            F[m].resize((size_t)rows[m] * r);
            for (auto& v : F[m])
                v = dist(gen);
        }
    }
    if (!init_file.empty()) {
        FILE* f = fopen(init_file.c_str(), "rb");
        size_t got = 0;
        for (int m = 0; m < 3 && f; m++)
            got += fread(F[m].data(), sizeof(double), F[m].size(), f);
        if (f)
            fclose(f);
        if (got != (size_t)(cfg.I + (int64_t)cfg.J + cfg.K) * r) {
            cerr << "Failed to read " << (int64_t)(cfg.I + (int64_t)cfg.J + cfg.K) * r << " initial values from "
                 << init_file << endl;
            return 1;
        }
    }

    // block_problem (block.cu:1233-1287)
    btc_schedule* sched = nullptr;
    if ((st = btc_schedule_build(&cfg, train.xyz, train.n, &sched)))
        fail(st, "block construction");
    btc_schedule_summary sm;
    btc_schedule_summarize(sched, &sm);
    cout << "max_parallel=" << sm.max_parallel_cf << " target_gpu_blocks=" << sm.target_gpu_blocks;
    if (cfg.parallel_sequence_size > 0)
        cout << " configured_parallel_sequence_size=" << cfg.parallel_sequence_size;
    cout << endl;
    std::ostringstream rs;
    rs << train_rate;
    string dir = output_root;
    if (!dir.empty() && dir[dir.size() - 1] != '/' && dir[dir.size() - 1] != '\\')
        dir += "/";
    dir += dataset_name + "_" + rs.str() + "/";
    if (!make_dirs(dir))
        cerr << "mkdir failed for " << dir << endl;
    string report = dir + "block_parallel.txt";
    if (btc_schedule_write_report(sched, &cfg, report.c_str()) != BTC_OK)
        cerr << "Failed to open " << report << endl;
    else
        cout << "block_parallel_report=" << report << endl;

    // sgd_train (sgd_Kernel.cu:968-1361)
    cout << "CUDA visible GPU count=" << ndev << endl;
    for (int d = 0; d < ndev; d++) {
        char name[256];
        int32_t smc = 0;
        int64_t mem = 0;
        if (btc_device_info(d, name, &smc, &mem) == BTC_OK)
            cout << "  GPU[" << d << "] name=\"" << name << "\" sm_count=" << smc
                 << " memory_MB=" << (unsigned long long)(mem / (1024LL * 1024LL)) << endl;
    }
    int active = cfg.requested_gpu_count == 0 ? ndev : std::min<int>(cfg.requested_gpu_count, ndev);
    if (cfg.requested_gpu_count > ndev)
        cout << "requested_gpus=" << cfg.requested_gpu_count << " exceeds visible GPU count; using " << active
             << " GPU(s)." << endl;
    if (active > 1)
        cout << "Training on one GPU; using GPU[" << cfg.device << "]." << endl;
    cout << "Using 1 GPU(s) for training." << endl;
    std::ofstream ofs_error((dir + "error.txt").c_str(), std::ios::out | std::ios::trunc);
    std::ofstream ofs_time((dir + "time.txt").c_str(), std::ios::out | std::ios::trunc);
    std::ofstream ofs_kernel((dir + "kernel_time.txt").c_str(), std::ios::out | std::ios::trunc);
    std::ofstream ofs_sync((dir + "sync_time.txt").c_str(), std::ios::out | std::ios::trunc);
    ofs_error << std::setprecision(10);
    ofs_error << "epoch test_RMSE test_MAE test_ER test_count" << endl;
    cout << "factor_matrix_bytes A=" << (size_t)cfg.I * r * 8 << " B=" << (size_t)cfg.J * r * 8
         << " C=" << (size_t)cfg.K * r * 8 << endl;

    btc_ctx* ctx = nullptr;
    if ((st = btc_ctx_create(&cfg, sched, train.xyz, train.val, train.n, test.xyz, test.val, test.n, &ctx)))
        fail(st, "device setup");
    for (int m = 0; m < 3; m++)
        if ((st = btc_ctx_set_factors(ctx, m, F[m].data())))
            fail(st, "factor upload");
    btc_metrics met;
    if (sm.num_slots > 0) {
        cout << sm.max_parallel << "   " << sm.num_slots << endl;
        // warm up the same kernel path once, then restore the factors
        btc_epoch_stats es;
        if ((st = btc_train_epoch(ctx, &es)))
            fail(st, "warm-up epoch");
        for (int m = 0; m < 3; m++)
            if ((st = btc_ctx_set_factors(ctx, m, F[m].data())))
                fail(st, "factor restore after warm-up");
        double prev = 0;
        int have_prev = 0;
        for (int epoch = 0; epoch < cfg.epochs; epoch++) {
            double t = now_s();
            if ((st = btc_train_epoch(ctx, &es)))
                fail(st, "epoch");
            t = now_s() - t;
            ofs_kernel << t << endl;
            ofs_sync << 0 << endl;
            ofs_time << t << endl;
            if ((st = btc_eval(ctx, BTC_SPLIT_TEST, &met)))
                fail(st, "metrics");
            ofs_error << epoch << ' ' << met.rmse << ' ' << met.mae << ' ' << met.er << ' ' << met.count << endl;
            // the lock-free loop prints no device prefix and stops at a 1e-7
            // improvement (sgd_Kernel.cu:1183-1191), the others at 1e-8
            // (sgd_Kernel.cu:1308-1317)
            const bool lockfree = cfg.mode == BTC_MODE_LOCKFREE;
            if (!lockfree)
                cout << "GPU:" << ndev << ' ';
            cout << "Epoch:" << epoch << " test_RMSE=" << met.rmse << '\n';
            if (have_prev && prev - met.rmse < (lockfree ? 0.0000001 : 0.00000001))
                break;
            prev = met.rmse;
            have_prev = 1;
        }
    }
    if ((st = btc_eval(ctx, BTC_SPLIT_TEST, &met)))
        fail(st, "metrics");
    cout << "Final test RMSE=" << met.rmse << " MAE=" << met.mae << " ER=" << met.er << " count=" << met.count
         << endl;
    for (int m = 0; m < 3; m++)
        if ((st = btc_ctx_get_factors(ctx, m, F[m].data())))
            fail(st, "factor download");
    btc_ctx_destroy(ctx);
    btc_schedule_free(sched);

    {
        const int32_t* e = train.xyz;
        double pred = 0;
        for (int q = 0; q < r; q++)
            pred += F[0][(size_t)e[0] * r + q] * F[1][(size_t)e[1] * r + q] * F[2][(size_t)e[2] * r + q];
        printf("first train entry: (%d,%d,%d) ref=%f pred=%f\n", e[0], e[1], e[2], train.val[0], pred);
    }
    if (!dump_dir.empty()) {
        if (!make_dirs(dump_dir))
            cerr << "mkdir failed for " << dump_dir << endl;
        const char* names[3] = {"A.txt", "B.txt", "C.txt"};
        for (int m = 0; m < 3; m++)
            write_factor(join_path(dump_dir, names[m]), F[m], rows[m], r);
    }
    return 0;
}
