// capi.cu -- extern "C" entry points of the ERI / J-K kernels and the error state.
#include <cstdarg>
#include <cstdio>

#include <mutex>

#include "capi_internal.cuh"
#include "eri.cuh"
#include "eri_warp.cuh"

namespace sq {

static thread_local char g_err[512] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int check_launch(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return SQ_OK;
}

#define DECL(QC) cudaError_t launch_qc_##QC(const EriArgs &, int, int, cudaStream_t);
DECL(0) DECL(1) DECL(2) DECL(3) DECL(4) DECL(5) DECL(6) DECL(7) DECL(8) DECL(9) DECL(10) DECL(11)
DECL(21) DECL(22) DECL(28)
#undef DECL
#define DECL32(QC) cudaError_t launch_qc_##QC##_f32(const EriArgs &, int, int, cudaStream_t);
DECL32(12) DECL32(13) DECL32(14) DECL32(15) DECL32(16) DECL32(17) DECL32(18)
#undef DECL32

// FP32 (SQ_FP32) per-thread kernels of the heavy classes.
static const eri_launcher kLaunchersF32[SQ_MAX_QCLASS] = {
    nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
    nullptr, nullptr, nullptr, nullptr, nullptr, launch_qc_12_f32, launch_qc_13_f32,
    launch_qc_14_f32, launch_qc_15_f32, launch_qc_16_f32, launch_qc_17_f32, launch_qc_18_f32, nullptr, nullptr,
};

// Classes with an f shell (eri_block.cu): one CTA per contracted quartet.
cudaError_t launch_eri_block(const EriArgs &, int, int, int, int, int, int, cudaStream_t);

#define DECL64(QC) cudaError_t launch_qc_##QC##_f64(const EriArgs &, int, int, cudaStream_t);
DECL64(12) DECL64(13) DECL64(14) DECL64(15) DECL64(16) DECL64(17) DECL64(18)
#undef DECL64
#define DECLDF(QC) cudaError_t launch_qc_##QC##_df(const EriArgs &, int, int, cudaStream_t);
DECLDF(0) DECLDF(1) DECLDF(2) DECLDF(3) DECLDF(4) DECLDF(5) DECLDF(6) DECLDF(7) DECLDF(8) DECLDF(9) DECLDF(10)
DECLDF(11) DECLDF(12) DECLDF(13) DECLDF(14) DECLDF(15) DECLDF(16) DECLDF(17) DECLDF(18)
#undef DECLDF

// Double-float (SQ_DF64) per-thread kernels of classes 0-18, (ss|ss) to
// (dd|ds): the classes of the s, p, d per-thread kernels.
static const eri_launcher kLaunchersDF[SQ_MAX_QCLASS] = {
    launch_qc_0_df,  launch_qc_1_df,  launch_qc_2_df,  launch_qc_3_df,  launch_qc_4_df,  launch_qc_5_df,
    launch_qc_6_df,  launch_qc_7_df,  launch_qc_8_df,  launch_qc_9_df,  launch_qc_10_df, launch_qc_11_df,
    launch_qc_12_df, launch_qc_13_df, launch_qc_14_df, launch_qc_15_df, launch_qc_16_df, launch_qc_17_df,
    launch_qc_18_df, nullptr,         nullptr,
};

// FP64 (SQ_FP64) per-thread kernels of classes 12-18, (dp|pp) to (dd|ds): their
// register blocks spill partly to local memory, and they still outrun the
// generic warp kernel.
static const eri_launcher kLaunchersF64[SQ_MAX_QCLASS] = {
    nullptr,          nullptr,          nullptr,          nullptr,          nullptr,          nullptr,
    nullptr,          nullptr,          nullptr,          nullptr,          nullptr,          nullptr,
    launch_qc_12_f64, launch_qc_13_f64, launch_qc_14_f64, launch_qc_15_f64, launch_qc_16_f64, launch_qc_17_f64,
    launch_qc_18_f64, nullptr,          nullptr,
};

// Per-thread (fully unrolled) J/K kernels exist for the light classes (L <= 4,
// except (dd|ss); with f: (fs|ss), (fs|ps), (fp|ss)) in every precision, and
// for classes 12-18 in SQ_FP64 and SQ_FP32.  Every other launch runs on the
// generic warp kernel when its blocks fit the warp kernel's tables (s, p, d
// shells, and bra pairs (fs), (fp): at most 36 components per pair, L <= 8),
// else on the block kernel ((fd|..), (ff|..)).
// SQ_OPT_GENERIC_MIN_L = 0 sends everything to it.
static const eri_launcher kLaunchers[SQ_MAX_QCLASS] = {
    launch_qc_0,  launch_qc_1,  launch_qc_2, launch_qc_3, launch_qc_4, launch_qc_5, launch_qc_6,
    launch_qc_7,  launch_qc_8,  launch_qc_9, launch_qc_10, launch_qc_11, nullptr, nullptr,
    nullptr,      nullptr,      nullptr,     nullptr,     nullptr,     nullptr,     nullptr,
    launch_qc_21, launch_qc_22, nullptr,     nullptr,     nullptr,     nullptr,     nullptr,
    launch_qc_28,
};

// Angular momenta of pair class pc (la >= lb).
static void pair_class_l(int pc, int &la, int &lb) {
    la = 0;
    while ((la + 1) * (la + 2) / 2 <= pc) ++la;
    lb = pc - la * (la + 1) / 2;
}

static void quartet_class_l(int qc, int &la, int &lb, int &lc, int &ld) {
    int cb = 0;
    while ((cb + 1) * (cb + 2) / 2 <= qc) ++cb;
    const int ck = qc - cb * (cb + 1) / 2;
    pair_class_l(cb, la, lb);
    pair_class_l(ck, lc, ld);
}

// Classes with la+lb+lc+ld >= g_generic_min_l use the warp kernel.
static int g_generic_min_l = 5;
// Bit c set: the FP64 J/K launches of class c run on its kLaunchersF64 kernel,
// else on the warp kernel (option SQ_OPT_FP64_UNROLLED_HIGH).
static long long g_fp64_unrolled_high = 0x7FLL << 12;  // classes 12-18
// Classes of SQ_DF64 launches on the double-float kernels (option SQ_OPT_DF_CLASSES):
// -1 the measured policy kDfPolicy, else a bit mask.
static long long g_df_classes = -1;
// Per class, measured on the (H2O)16 cc-pVDZ lists against the FP64 kernels:
// 2 double-float is faster at any launch length; 1 only on long launches
// (throughput-bound; a short launch is bound by one thread's latency, and a
// double-float operation is a longer dependent chain than one FP64 FMA);
// 0 never (the double-float kernel spills more than the FP64 one).
static const signed char kDfPolicy[SQ_MAX_QCLASS] = {2, 2, 2, 2, 1, 1, 2, 2, 1, 1, 2, 1, 0, 0, 0, 2, 2, 0, 0};
static bool df_class(int c, long long nq) {
    if (g_df_classes >= 0) return (g_df_classes >> c) & 1;
    return kDfPolicy[c] == 2 || (kDfPolicy[c] == 1 && nq >= 512LL * sm_count());
}
// Per-thread gradient kernels for the light classes (option SQ_OPT_GRAD_THREAD).
static int g_grad_thread = 1;
int grad_thread_enabled() { return g_grad_thread; }

// Autotuned launch shapes per (quartet class, precision); threads 0 = default.
struct LaunchCfg {
    int threads;
    long long blocks;
};
static LaunchCfg g_cfg[SQ_MAX_QCLASS][3] = {};

static int check_common(const char *who, const sq_basis *basis, const sq_pairs *pairs, const sq_quartets *qs,
                        const double *tab) {
    if (!basis || !pairs || !qs || !tab) return set_error(SQ_ERR_ARG, "%s: NULL argument", who);
    if (!pairs->prim || !pairs->herm || !pairs->pp_off || !pairs->herm_off || !pairs->shells)
        return set_error(SQ_ERR_ARG, "%s: pair data not allocated", who);
    if (qs->nquartet < 0 || qs->class_off[0] != 0 || qs->class_off[SQ_MAX_QCLASS] != qs->nquartet)
        return set_error(SQ_ERR_ARG, "%s: quartet class offsets inconsistent", who);
    for (int c = 0; c < SQ_MAX_QCLASS; ++c)
        if (qs->class_off[c + 1] < qs->class_off[c])
            return set_error(SQ_ERR_ARG, "%s: quartet class offsets not ascending", who);
    if (qs->nquartet > 0 && !qs->pairs) return set_error(SQ_ERR_ARG, "%s: quartet list is NULL", who);
    return SQ_OK;
}

// J/K class launches are independent (every contribution is an atomic add),
// so they are spread over a small pool of streams forked from and joined back
// into the caller's stream: the tail of one class overlaps the start of the
// next.  g_jk_streams = 1 keeps every launch on the caller's stream.
// Successive calls take the next streams of the pool (round robin), so two
// calls issued from different caller streams (the FP64 and FP32 lists of a
// mixed build) do not queue behind each other.
static int g_jk_streams = 8;
constexpr int kMaxPoolStreams = 16;
constexpr int kMaxPoolDevices = 64;

struct StreamPool {
    bool ready = false;
    int next = 0;
    cudaStream_t s[kMaxPoolStreams];
    cudaEvent_t fork[kMaxPoolStreams];
    cudaEvent_t join[kMaxPoolStreams];
};
static StreamPool g_pool[kMaxPoolDevices];
static std::mutex g_pool_mutex;

// Caller holds g_pool_mutex.
static int pool_for_current_device(StreamPool **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "stream pool: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxPoolDevices) return set_error(SQ_ERR_ARG, "stream pool: device %d out of range", dev);
    StreamPool &p = g_pool[dev];
    if (!p.ready) {
        e = cudaSuccess;
        for (int i = 0; i < kMaxPoolStreams && e == cudaSuccess; ++i) {
            e = cudaStreamCreateWithFlags(&p.s[i], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.fork[i], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.join[i], cudaEventDisableTiming);
        }
        if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "stream pool: %s", cudaGetErrorString(e));
        p.ready = true;
    }
    *out = &p;
    return SQ_OK;
}

static cudaError_t launch_class(EriArgs &args, const sq_quartets *qs, int c, int mode, int precision,
                                cudaStream_t stream) {
    args.quartets = reinterpret_cast<const int2 *>(qs->pairs) + qs->class_off[c];
    args.nq = qs->class_off[c + 1] - qs->class_off[c];
    int la, lb, lc, ld;
    quartet_class_l(c, la, lb, lc, ld);
    if (mode == MODE_JK && precision >= 0 && precision <= SQ_FP64_PRIM) {
        const int pi = precision == SQ_FP64_PRIM ? SQ_FP64 : precision;
        args.cfg_threads = g_cfg[c][pi].threads;
        args.cfg_blocks = g_cfg[c][pi].blocks;
    } else {
        args.cfg_threads = 0;
        args.cfg_blocks = 0;
    }
    const int L = la + lb + lc + ld;
    const bool warp_fits = ncart(la) * ncart(lb) <= ncart(SQ_LMAX) * ncart(SQ_LMAX) &&
                           ncart(lc) * ncart(ld) <= ncart(SQ_LMAX) * ncart(SQ_LMAX) && L <= 4 * SQ_LMAX;
    eri_launcher unrolled = nullptr;
    if (mode == MODE_JK && L < g_generic_min_l) unrolled = kLaunchers[c];
    if (mode == MODE_JK && precision == SQ_FP32 && kLaunchersF32[c] != nullptr && g_generic_min_l > 0)
        unrolled = kLaunchersF32[c];
    if (mode == MODE_JK && (precision == SQ_FP64 || precision == SQ_FP64_PRIM) && kLaunchersF64[c] != nullptr &&
        g_generic_min_l > 0 && ((g_fp64_unrolled_high >> c) & 1))
        unrolled = kLaunchersF64[c];
    // SQ_DF64 runs on the double-float kernels where a class has one, else as
    // SQ_FP64_PRIM (which keeps the per-thread f classes' split)
    if (mode == MODE_JK && precision == SQ_DF64) {
        if (kLaunchersDF[c] != nullptr && g_generic_min_l > 0 && df_class(c, args.nq))
            return kLaunchersDF[c](args, mode, precision, stream);
        return launch_class(args, qs, c, mode, SQ_FP64_PRIM, stream);
    }
    // SQ_FP64_PRIM reaches only the per-thread kernels of kLaunchers; every
    // other kernel runs such a launch as plain FP64
    const int plain = precision == SQ_FP64_PRIM ? SQ_FP64 : precision;
    if (mode == MODE_JK && precision == SQ_FP64_PRIM && L < g_generic_min_l && kLaunchers[c] != nullptr)
        return kLaunchers[c](args, mode, precision, stream);
    if (unrolled != nullptr) return unrolled(args, mode, plain, stream);
    if (!warp_fits) return launch_eri_block(args, la, lb, lc, ld, mode, plain, stream);
    // FP32 J/K launches on the warp kernel evaluate each lane's F_m by its own
    // FP32 Taylor expansion: there is no recursion to carry FP32 errors, and the
    // FP64 expansion (seven DFMAs per lane and primitive quartet) cost the f
    // classes' FP32 launches about 10 %.  The FP32 table reaches m = 10 (the
    // warp kernel: L <= 8).
    const int warp_prec = (mode == MODE_JK && plain == SQ_FP32 && L <= SQ_BOYS_NCOL - 1 - kBoysTaylor32)
                              ? SQ_FP32_BOYS32
                              : plain;
    return launch_eri_warp(args, WarpClass{la, lb, lc, ld}, mode, warp_prec, stream);
}

static int run_classes(const char *who, EriArgs args, const sq_quartets *qs, int mode, int precision,
                       cudaStream_t stream, bool pooled = true) {
    int nonempty = 0;
    for (int c = 0; c < SQ_MAX_QCLASS; ++c) nonempty += qs->class_off[c + 1] > qs->class_off[c];
    const int nstream = !pooled ? 1 : (g_jk_streams < nonempty ? g_jk_streams : nonempty);
    if (mode == MODE_JK && nstream > 1) {
        std::lock_guard<std::mutex> lock(g_pool_mutex);
        StreamPool *pool = nullptr;
        int rc = pool_for_current_device(&pool);
        if (rc) return rc;
        const int first = pool->next;
        pool->next = (pool->next + nstream) % kMaxPoolStreams;
        auto sid = [&](int i) { return (first + i) % kMaxPoolStreams; };
        cudaError_t e = cudaEventRecord(pool->fork[first], stream);
        for (int i = 0; i < nstream && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(pool->s[sid(i)], pool->fork[first], 0);
        // classes in index order (light, many-quartet classes first, the few
        // high-L classes last), round robin over the streams; ordering by an
        // estimate of each launch's work queued the heavy classes behind the
        // long-running high-L ones on the same streams and measured slower
        int k = 0;
        for (int c = 0; c < SQ_MAX_QCLASS && e == cudaSuccess; ++c) {
            if (qs->class_off[c + 1] == qs->class_off[c]) continue;
            e = launch_class(args, qs, c, mode, precision, pool->s[sid(k++ % nstream)]);
            if (e != cudaSuccess) {
                set_error(SQ_ERR_CUDA, "%s: class %d: %s", who, c, cudaGetErrorString(e));
                break;
            }
        }
        // always join what was forked, so the caller's stream (or a capture) stays whole
        for (int i = 0; i < nstream; ++i) {
            cudaError_t ej = cudaEventRecord(pool->join[sid(i)], pool->s[sid(i)]);
            if (ej == cudaSuccess) ej = cudaStreamWaitEvent(stream, pool->join[sid(i)], 0);
            if (e == cudaSuccess) e = ej;
        }
        if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "%s: %s", who, cudaGetErrorString(e));
        return SQ_OK;
    }
    for (int c = 0; c < SQ_MAX_QCLASS; ++c) {
        if (qs->class_off[c + 1] == qs->class_off[c]) continue;
        const cudaError_t e = launch_class(args, qs, c, mode, precision, stream);
        if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "%s: class %d: %s", who, c, cudaGetErrorString(e));
    }
    return SQ_OK;
}

}  // namespace sq

using namespace sq;

extern "C" int sq_version(void) { return 1; }

extern "C" const char *sq_last_error(void) { return g_err; }

extern "C" int sq_set_option(int key, long long value) {
    if (key == SQ_OPT_JK_STREAMS) {
        if (value < 1 || value > kMaxPoolStreams)
            return set_error(SQ_ERR_ARG, "sq_set_option: J/K streams must be 1..%d", kMaxPoolStreams);
        g_jk_streams = (int)value;
        return SQ_OK;
    }
    if (key == SQ_OPT_GRAD_THREAD) {
        g_grad_thread = value != 0;
        return SQ_OK;
    }
    if (key == SQ_OPT_FP64_UNROLLED_HIGH) {
        if (value < 0 || value >= (1LL << SQ_MAX_QCLASS))
            return set_error(SQ_ERR_ARG, "sq_set_option: class mask out of range");
        g_fp64_unrolled_high = value;
        return SQ_OK;
    }
    if (key == SQ_OPT_DF_CLASSES) {
        if (value < -1 || value >= (1LL << SQ_MAX_QCLASS))
            return set_error(SQ_ERR_ARG, "sq_set_option: class mask out of range");
        g_df_classes = value;
        return SQ_OK;
    }
    if (key == SQ_OPT_GENERIC_MIN_L) {
        if (value < 0) return set_error(SQ_ERR_ARG, "sq_set_option: negative L");
        g_generic_min_l = (int)value;
        return SQ_OK;
    }
    return set_error(SQ_ERR_ARG, "sq_set_option: unknown key %d", key);
}

extern "C" int sq_set_launch_config(int qclass, int precision, int threads, long long max_blocks) {
    if (qclass < 0 || qclass >= SQ_MAX_QCLASS || precision < 0 || precision > 2)
        return set_error(SQ_ERR_ARG, "sq_set_launch_config: bad class %d / precision %d", qclass, precision);
    if (threads != 0 && (threads < 32 || threads > 128 || threads % 32 != 0 || max_blocks < 1))
        return set_error(SQ_ERR_ARG, "sq_set_launch_config: threads must be 32..128 (multiple of 32), blocks >= 1");
    g_cfg[qclass][precision] = LaunchCfg{threads, threads ? max_blocks : 0};
    return SQ_OK;
}

extern "C" long long sq_get_option(int key) {
    if (key == SQ_OPT_GENERIC_MIN_L) return g_generic_min_l;
    if (key == SQ_OPT_JK_STREAMS) return g_jk_streams;
    if (key == SQ_OPT_FP64_UNROLLED_HIGH) return g_fp64_unrolled_high;
    if (key == SQ_OPT_GRAD_THREAD) return g_grad_thread;
    if (key == SQ_OPT_DF_CLASSES) return g_df_classes;
    return -1;
}

extern "C" int sq_schwarz(const sq_basis *basis, const sq_pairs *pairs, const sq_quartets *diagonal,
                          const double *table64, double *q, void *stream) {
    int rc = check_common("sq_schwarz", basis, pairs, diagonal, table64);
    if (rc) return rc;
    if (!q) return set_error(SQ_ERR_ARG, "sq_schwarz: q is NULL");
    EriArgs a{};
    a.basis = *basis;
    a.pairs = *pairs;
    a.tab64 = table64;
    a.q = q;
    return run_classes("sq_schwarz", a, diagonal, MODE_SCHWARZ, SQ_FP64, (cudaStream_t)stream);
}

extern "C" int sq_eri_dense(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots,
                            const sq_quartets *quartets, const double *table64, double *V, void *stream) {
    int rc = check_common("sq_eri_dense", basis, pairs, quartets, table64);
    if (rc) return rc;
    if (!V) return set_error(SQ_ERR_ARG, "sq_eri_dense: V is NULL");
    EriArgs a{};
    a.basis = *basis;
    a.pairs = *pairs;
    if (slots) {
        a.slots = *slots;
        a.use_slots = 1;
    }
    a.tab64 = table64;
    a.V = V;
    return run_classes("sq_eri_dense", a, quartets, MODE_DENSE, SQ_FP64, (cudaStream_t)stream);
}

static int jk_common(const char *who, const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots,
                     const sq_quartets *quartets, const double *table64, const float *table32, int nd,
                     const double *D, float *D32, double *Jacc, double *Kacc, int precision, void *stream,
                     bool pooled = true, float prim_tau = 0.0f, float *Ddf = nullptr) {
    int rc = check_common(who, basis, pairs, quartets, table64);
    if (rc) return rc;
    if (!slots || !slots->prim || !slots->herm || !slots->pair || !slots->desc)
        return set_error(SQ_ERR_ARG, "%s: slot layout with descriptors (sq_slots_describe) is required", who);
    if (basis->mat_base != nullptr && !slots->mbase)
        return set_error(SQ_ERR_ARG, "%s: a packed batch basis needs slots->mbase", who);
    if (!D || !Jacc || !Kacc) return set_error(SQ_ERR_ARG, "%s: D, Jacc and Kacc are required", who);
    if (nd < 1) return set_error(SQ_ERR_ARG, "%s: nd = %d densities", who, nd);
    if (precision != SQ_FP64 && precision != SQ_FP32 && precision != SQ_FP32_BOYS32 && precision != SQ_FP64_PRIM &&
        precision != SQ_DF64)
        return set_error(SQ_ERR_ARG, "%s: unknown precision %d", who, precision);
    if ((precision == SQ_FP64_PRIM || precision == SQ_DF64) &&
        ((prim_tau > 0.0f && !pairs->pq) || !slots->prim32v || !slots->herm32 || !table32 || !(prim_tau >= 0.0f)))
        return set_error(SQ_ERR_ARG, "%s: primitive-level precision needs FP32 slot data, table32, a non-negative "
                         "bound and, for a bound above zero, pairs->pq", who);
    if (precision == SQ_DF64 && (!Ddf || !slots->primdf || !slots->hermdf))
        return set_error(SQ_ERR_ARG, "%s: double-float launches need Ddf and slots->primdf, slots->hermdf", who);
    cudaStream_t s = (cudaStream_t)stream;
    const long long mt = mat_total(*basis);
    if (mt >= (1LL << 31))
        return set_error(SQ_ERR_ARG, "%s: %lld matrix elements exceed the kernels' 32-bit indexing", who, mt);
    if (precision == SQ_DF64) {
        rc = to_df(mt * nd, D, Ddf, s);
        if (rc) return rc;
    }
    if (precision != SQ_FP64 && precision != SQ_FP64_PRIM && precision != SQ_DF64) {
        if (!D32 || !pairs->prim32 || !pairs->herm32 || !slots->prim32 || !slots->herm32 || !slots->prim32v ||
            !table32)
            return set_error(SQ_ERR_ARG, "%s: FP32 precision needs D32, FP32 pair/slot data and table32", who);
        rc = to_float(mt * nd, D, D32, s);
        if (rc) return rc;
    }
    EriArgs a{};
    a.nd = nd;
    a.dstride = mt;
    a.basis = *basis;
    a.pairs = *pairs;
    a.tab64 = table64;
    a.tab32 = table32;
    a.D = D;
    a.D32 = D32;
    a.slots = *slots;
    a.use_slots = 1;
    a.Jacc = Jacc;
    a.Kacc = Kacc;
    a.prim_tau = prim_tau;
    a.Ddf = Ddf;
    return run_classes(who, a, quartets, MODE_JK, precision, s, pooled);
}

// sq_jk with every class launch on the caller's stream: no library streams or
// events are created (the allocation-free entry point uses it).
int sq::jk_serial(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
              const double *table64, const float *table32, const double *D, float *D32, double *Jacc, double *Kacc,
              int precision, void *stream) {
    return jk_common("sq_jk_noalloc", basis, pairs, slots, quartets, table64, table32, 1, D, D32, Jacc, Kacc,
                     precision, stream, false);
}

extern "C" int sq_jk(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots,
                     const sq_quartets *quartets, const double *table64, const float *table32, const double *D,
                     float *D32, double *Jacc, double *Kacc, int precision, void *stream) {
    return jk_common("sq_jk", basis, pairs, slots, quartets, table64, table32, 1, D, D32, Jacc, Kacc, precision,
                     stream);
}

extern "C" int sq_jk_prim(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots,
                          const sq_quartets *quartets, const double *table64, const float *table32, const double *D,
                          double *Jacc, double *Kacc, double prim_tau, void *stream) {
    return jk_common("sq_jk_prim", basis, pairs, slots, quartets, table64, table32, 1, D, nullptr, Jacc, Kacc,
                     SQ_FP64_PRIM, stream, true, (float)prim_tau);
}

extern "C" int sq_jk_df(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots,
                        const sq_quartets *quartets, const double *table64, const float *table32, const double *D,
                        float *Ddf, double *Jacc, double *Kacc, double prim_tau, void *stream) {
    return jk_common("sq_jk_df", basis, pairs, slots, quartets, table64, table32, 1, D, nullptr, Jacc, Kacc,
                     SQ_DF64, stream, true, (float)prim_tau, Ddf);
}

extern "C" int sq_df_class(int qclass, long long nquartets) {
    if (qclass < 0 || qclass >= SQ_MAX_QCLASS) return 0;
    return kLaunchersDF[qclass] != nullptr && g_generic_min_l > 0 && df_class(qclass, nquartets);
}

extern "C" int sq_jk_multi(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots,
                           const sq_quartets *quartets, const double *table64, const float *table32, int nd,
                           const double *D, float *D32, double *Jacc, double *Kacc, int precision, void *stream) {
    return jk_common("sq_jk_multi", basis, pairs, slots, quartets, table64, table32, nd, D, D32, Jacc, Kacc,
                     precision, stream);
}
