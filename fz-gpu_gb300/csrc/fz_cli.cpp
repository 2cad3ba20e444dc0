// fz-gpu -- drop-in for the reference CLI (fz.cu:226-238 main, fz.cu:113-224 runSzs).
//
//   fz-gpu <path> <x> <y> <z> <rel_eb> [-o stream.fz] [--compat] [--json]
//       Compresses the float32 file at <path> (x fastest; the element count comes from
//       the file size, fz.cu:117-118) with a relative error bound and prints the
//       reference's three lines (fz.cu:207-209).  -o writes the stream to a file.
//   fz-gpu --decompress <stream.fz> -o <out.f32> [--verify <orig.f32>] [--json]
//       Reconstructs the field; --verify prints max |x - x'| and PSNR (verify.hh:24-83).
//
// Errors print one line to stderr and exit non-zero (the reference exits 1 or
// EXIT_FAILURE, fz.cu:30-33, cuda_err.cuh:31-173).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fz.h"

namespace {

// The reference has no outlier channel (its codes are 16 bits): deltas that do not fit
// are reported, on stderr so that stdout keeps the reference's three lines.
void warn_overflow(const fz_header& h)
{
    if (h.flags & FZ_FLAG_CODE_OVERFLOW)
        std::fprintf(stderr,
                     "warning: some prediction deltas do not fit the 16-bit codes (|delta| >= 2^15, or "
                     "non-finite input); the stream does not meet the error bound at those points "
                     "(FZ_FLAG_CODE_OVERFLOW)\n");
}

int die(const char* what, fz_status st)
{
    std::fprintf(stderr, "fz-gpu: %s: %s\n", what, fz_status_string(st));
    return 1;
}

bool read_file(const std::string& path, std::vector<char>& buf)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(sz > 0 ? (size_t)sz : 0);
    size_t got = buf.empty() ? 0 : std::fread(buf.data(), 1, buf.size(), f);
    std::fclose(f);
    return got == buf.size();
}

bool write_file(const std::string& path, const void* p, size_t n)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    size_t put = std::fwrite(p, 1, n, f);
    std::fclose(f);
    return put == n;
}

void usage()
{
    std::fprintf(stderr,
                 "usage: fz-gpu <path> <x> <y> <z> <rel_eb> [-o stream.fz] [--compat] [--json]\n"
                 "       fz-gpu --decompress <stream.fz> -o <out.f32> [--verify <orig.f32>] [--json]\n");
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int decompress_main(int argc, char** argv)
{
    std::string in, out, verify;
    bool        json = false;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--decompress") && i + 1 < argc) in = argv[++i];
        else if (!std::strcmp(argv[i], "-o") && i + 1 < argc) out = argv[++i];
        else if (!std::strcmp(argv[i], "--verify") && i + 1 < argc) verify = argv[++i];
        else if (!std::strcmp(argv[i], "--json")) json = true;
        else {
            usage();
            return 2;
        }
    }
    if (in.empty() || out.empty()) {
        usage();
        return 2;
    }
    std::vector<char> st;
    if (!read_file(in, st) || st.size() < FZ_HEADER_BYTES) {
        std::fprintf(stderr, "fail to open %s\n", in.c_str());
        return 1;
    }
    fz_header h;
    std::memcpy(&h, st.data(), sizeof(h));
    uint64_t need = 0;
    fz_status s = fz_stream_bytes(&h, &need);
    if (s != FZ_SUCCESS || need > st.size()) return die("stream", s != FZ_SUCCESS ? s : FZ_CORRUPT_STREAM);
    fz_workspace* ws = nullptr;
    if ((s = fz_workspace_create(h.n, &ws)) != FZ_SUCCESS) return die("workspace", s);
    void*  h_st  = nullptr;
    float* h_out = nullptr;
    cudaMallocHost(&h_st, st.size());
    cudaMallocHost((void**)&h_out, h.n * 4);
    std::memcpy(h_st, st.data(), st.size());
    double t0 = now_s();
    s         = fz_decompress_host(ws, h_st, st.size(), h_out, h.n, nullptr);
    double t1 = now_s();
    if (s != FZ_SUCCESS) return die("decompress", s);
    warn_overflow(h);
    if (!write_file(out, h_out, h.n * 4)) {
        std::fprintf(stderr, "fail to write %s\n", out.c_str());
        return 1;
    }
    double max_err = 0, psnr = 0;
    if (!verify.empty()) {
        std::vector<char> o;
        if (!read_file(verify, o) || o.size() / 4 != h.n) {
            std::fprintf(stderr, "fail to open %s\n", verify.c_str());
            return 1;
        }
        const float* x  = reinterpret_cast<const float*>(o.data());
        double       mn = x[0], mx = x[0], se = 0;
        for (uint64_t i = 0; i < h.n; ++i) {
            double e = std::fabs((double)h_out[i] - x[i]);
            max_err  = e > max_err ? e : max_err;
            se += e * e;
            mn = x[i] < mn ? x[i] : mn;
            mx = x[i] > mx ? x[i] : mx;
        }
        double mse = se / (double)h.n;
        psnr       = 20 * std::log10(mx - mn) - 10 * std::log10(mse);
        std::printf("max abs error: %g (eb %g, ratio %.6f)\nPSNR: %f\n", max_err, h.eb_abs,
                    max_err / h.eb_abs, psnr);
    }
    if (json)
        std::fprintf(stderr, "{\"decompress_s\": %.6f, \"n\": %llu, \"gbs\": %.3f}\n", t1 - t0,
                     (unsigned long long)h.n, 4.0 * h.n / (t1 - t0) / 1e9);
    fz_workspace_destroy(ws);
    cudaFreeHost(h_st);
    cudaFreeHost(h_out);
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    for (int i = 1; i < argc; ++i)
        if (!std::strcmp(argv[i], "--decompress")) return decompress_main(argc, argv);
    if (argc < 6) {
        usage();
        return 2;
    }
    const std::string path = argv[1];
    fz_dims           dims;
    char*             end = nullptr;
    long              x = std::strtol(argv[2], &end, 10), y = std::strtol(argv[3], nullptr, 10),
         z        = std::strtol(argv[4], nullptr, 10);
    const double eb = std::strtod(argv[5], nullptr);
    std::string  out;
    bool         json = false;
    fz_mode      mode = FZ_MODE_SIDECAR;
    for (int i = 6; i < argc; ++i) {
        if (!std::strcmp(argv[i], "-o") && i + 1 < argc) out = argv[++i];
        else if (!std::strcmp(argv[i], "--json")) json = true;
        else if (!std::strcmp(argv[i], "--compat")) mode = FZ_MODE_COMPAT;
        else {
            usage();
            return 2;
        }
    }
    if (x <= 0 || y <= 0 || z <= 0) {
        usage();
        return 2;
    }
    dims.x = (uint32_t)x, dims.y = (uint32_t)y, dims.z = (uint32_t)z;

    std::vector<char> raw;
    if (!read_file(path, raw)) {
        std::fprintf(stderr, "fail to open %s\n", path.c_str());  // fz.cu:31
        return 1;
    }
    const uint64_t file_bytes = raw.size();
    const uint64_t n          = file_bytes / sizeof(float);  // fz.cu:118
    fz_workspace*  ws         = nullptr;
    fz_status      s          = fz_workspace_create(n ? n : 1, &ws);
    if (s != FZ_SUCCESS) return die("workspace", s);
    uint64_t cap = 0;
    if ((s = fz_max_compressed_bytes(n, dims, mode, &cap)) != FZ_SUCCESS) return die("arguments", s);
    float* h_in  = nullptr;
    void*  h_out = nullptr;
    cudaMallocHost((void**)&h_in, n * 4);
    cudaMallocHost(&h_out, cap);
    std::memcpy(h_in, raw.data(), n * 4);
    uint64_t bytes = 0;
    double   t0    = now_s();
    s = fz_compress_host(ws, h_in, n, dims, eb, FZ_EB_REL, mode, h_out, cap, &bytes, nullptr);
    double t1 = now_s();
    if (s != FZ_SUCCESS) return die("compress", s);
    fz_header h;
    std::memcpy(&h, h_out, sizeof(h));
    uint64_t orig = 0, comp = 0;
    double   ratio = 0;
    fz_reference_sizes(file_bytes, h.nnz, &orig, &comp, &ratio);
    // fz.cu:207-209, printed with the reference's formats
    std::printf("original size: %d\n", (int)orig);
    std::printf("compressed size: %d\n", (int)comp);
    std::printf("compression ratio: %f\n", (float)file_bytes / (float)comp);
    warn_overflow(h);
    if (!out.empty() && !write_file(out, h_out, bytes)) {
        std::fprintf(stderr, "fail to write %s\n", out.c_str());
        return 1;
    }
    if (json)
        std::fprintf(stderr,
                     "{\"stream_bytes\": %llu, \"nnz\": %llu, \"flags\": %u, \"compress_s\": %.6f, "
                     "\"gbs\": %.3f}\n",
                     (unsigned long long)bytes, (unsigned long long)h.nnz, h.flags, t1 - t0,
                     4.0 * n / (t1 - t0) / 1e9);
    fz_workspace_destroy(ws);
    cudaFreeHost(h_in);
    cudaFreeHost(h_out);
    return 0;
}
