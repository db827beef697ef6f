// ccsd_gemm_noalloc: the split-precision tensor-core contraction with all of
// its scratch in one fixed device array, so the call itself allocates nothing.
//
// Who needs it: callers that may not call cudaMalloc/cudaFree -- a process
// whose device memory is owned by another allocator with a fixed budget (a
// framework's caching allocator, a serving runtime that reserves all of HBM
// at start-up), and callers in the middle of a pipelined stream that cannot
// afford the device-wide synchronisation cudaFree implies.  ccsd_gemm
// allocates its split planes and workspace per call; this variant carves them
// out of g_arena instead.
//
// The arena is a file-scope static __device__ array of kArenaBytes (64 MiB):
// every GPU that loads the library holds it until the process exits.  Host
// code cannot use the symbol g_arena as a device address (on the host it is a
// stand-in object); the first call on each device resolves the real address
// with cudaGetSymbolAddress while that device is current and caches it.
// Every call reuses the same arena, so the contents left by the previous call
// are stale: the error word is cleared and the row maxima are re-zeroed on
// each call, and the planes/scales/partials are fully rewritten before use.
// Two calls whose work overlaps on the GPU (different streams, or different
// host threads on one device) race on the arena.
#include <mutex>
#include <string>
#include <utility>

#include "../../include/ccsd_gb300.h"
#include "split_gemm.h"

namespace ccsd {

void set_last_error(const std::string &msg);

namespace {

constexpr size_t kArenaBytes = 64ull << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_arena[kArenaBytes];

std::mutex g_arena_mu;
void *g_arena_addr[kMaxDevices] = {};

// Device address of g_arena on the current device (set up once per device).
unsigned char *arena_on_current_device() {
    int dev = 0;
    CCSD_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw Error(CCSD_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lock(g_arena_mu);
    if (!g_arena_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_arena);
        if (e != cudaSuccess || !p)
            throw Error(CCSD_ERR_CUDA, std::string("cudaGetSymbolAddress(g_arena) failed: ") + cudaGetErrorString(e));
        g_arena_addr[dev] = p;
    }
    return (unsigned char *)g_arena_addr[dev];
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Carve one split operand (planes, scales, row maxima) out of the arena.
void carve(SplitOperand &op, unsigned char *base, size_t &off, int rows, int K, int nslices) {
    op.rows = rows;
    op.rows_pad = (rows + 127) / 128 * 128;
    op.K = K;
    op.kpad = (K + 31) / 32 * 32;
    op.nslices = nslices;
    op.bytes = (size_t)nslices * op.rows_pad * op.kpad * 2;
    op.scale_cap = op.rows_pad;
    off = align256(off);
    op.planes = base + off;
    off += op.bytes;
    off = align256(off);
    op.scale = (double *)(base + off);
    off += sizeof(double) * op.rows_pad;
    off = align256(off);
    op.rmax = (unsigned long long *)(base + off);
    off += sizeof(unsigned long long) * op.rows_pad;
}

size_t operand_bytes(int rows, int K, int nslices) {
    const size_t rp = (size_t)(rows + 127) / 128 * 128, kp = (size_t)(K + 31) / 32 * 32;
    return align256((size_t)nslices * rp * kp * 2) + 2 * align256(8 * rp) + 256;
}

}  // namespace
}  // namespace ccsd

extern "C" int ccsd_gemm_noalloc(int32_t precision, int32_t M, int32_t N, int32_t K, double alpha,
                                 const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                                 double *C, int64_t ldc, void *stream) {
    using namespace ccsd;
    try {
        if (M < 0 || N < 0 || K < 0 || !A || !B || !C || lda < K || ldb < K || ldc < N)
            throw Error(CCSD_ERR_INVALID_ARG, "ccsd_gemm_noalloc: bad shape, leading dimension or NULL pointer");
        if (precision != CCSD_PREC_SPLIT2 && precision != CCSD_PREC_SPLIT3 && precision != CCSD_PREC_SPLIT4)
            throw Error(CCSD_ERR_INVALID_ARG, "ccsd_gemm_noalloc: precision must be CCSD_PREC_SPLIT2/3/4");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw Error(CCSD_ERR_NO_DEVICE, "no CUDA device: this engine has no CPU path");
        }
        if (M == 0 || N == 0) return CCSD_OK;
        cudaStream_t st = (cudaStream_t)stream;
        MatView a, b;
        a.p = A;
        a.row.s2 = lda;
        a.col.s2 = 1;
        b.p = B;
        b.row.s2 = ldb;
        b.col.s2 = 1;
        OutView c;
        c.p = C;
        c.row.s2 = ldc;
        c.col.s2 = 1;
        if (K == 0) {  // C = beta C, nothing to contract (alpha is not applied, as in BLAS)
            if (beta != 1.0) {
                MatView cv;
                cv.p = C;
                cv.row = c.row;
                cv.col = c.col;
                axpby_view(M, N, 0.0, cv, beta, c, st);
                CCSD_CUDA(cudaStreamSynchronize(st));
            }
            return CCSD_OK;
        }
        // the same operand roles as ccsd_gemm (SplitEngine::gemm): the long side in the
        // 128-row tile, and C's index with the smaller stride in the TMEM lanes
        if (SplitEngine::prefer_swap(M, N, c)) {
            std::swap(a, b);
            std::swap(M, N);
            std::swap(c.row, c.col);
        }
        const size_t need = 256 + operand_bytes(M, K, precision) + operand_bytes(N, K, precision);
        if (need > kArenaBytes)
            throw Error(CCSD_ERR_INVALID_ARG,
                        "ccsd_gemm_noalloc: operands need " + std::to_string(need) +
                            " bytes of scratch; the static arena holds " + std::to_string(kArenaBytes) +
                            " bytes (64 MiB) -- use ccsd_gemm for this size");
        unsigned char *base = arena_on_current_device();
        size_t off = 0;
        int *d_err = (int *)base;
        off = 256;
        SplitOperand opa, opb;
        carve(opa, base, off, M, K, precision);
        carve(opb, base, off, N, K, precision);
        off = align256(off);
        double *ws = (double *)(base + off);
        const size_t ws_elems = (kArenaBytes - off) / sizeof(double);
        CCSD_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st));
        split_operand_kernel_launch(opa, M, K, a, st);
        split_operand_kernel_launch(opb, N, K, b, st);
        split_gemm_launch(opa, opb, M, N, alpha, beta, c, ws, ws_elems, d_err, st);
        int herr = 0;
        CCSD_CUDA(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CCSD_CUDA(cudaStreamSynchronize(st));
        if (herr)
            throw Error(CCSD_ERR_TIMEOUT,
                        "ccsd_gemm_noalloc: a bounded device wait gave up (error word " + std::to_string(herr) + ")");
        return CCSD_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return CCSD_ERR_CUDA;
    }
}
