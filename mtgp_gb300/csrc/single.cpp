// single.cpp -- single generators (mtgp32_gpu_t / mtgp64_gpu_t): seeding,
// fills (split over many CTAs from windows jumped ahead when long), skips,
// jumps, export and import, and their entry points of the C ABI.
#include "host_internal.h"

namespace {

// n successive values of one generator.  A fill of at least kSplitFillMin
// values, on an exponent with GF(2) jumps, is cut into chunks: chunk c starts
// from the generator's window jumped by X^(c * chunk) mod chi.  Those windows
// are made first, every jump's correlation split over several CTAs
// (k_jump_part, a range of the jump kernel's tap chunks each), from
// polynomials kept on the device for the chunk length; then one batched
// launch runs every chunk from its window on the two-word core, with no jump
// inside it, and the window after the last chunk becomes the generator's.
// A 2^20-value fill takes 0.05 ms this way (0.12 ms with one in-kernel jump
// per chunk, 0.41 ms on one CTA), 2^26 values 0.18 ms.  Smaller fills,
// and fills issued while the stream is being captured, run on one CTA.  The
// first split fill of a parameter set also computes its characteristic
// polynomial and jump tables (tens of milliseconds, and a device
// synchronisation), and a new chunk length its chunk polynomials.
constexpr size_t kSplitFillMin = size_t(1) << 20;
constexpr int64_t kMaxFillChunks = 4096;

// Chunk length of a split fill of n values: the power of two nearest to
// 32 sqrt(n) for MEXP 11213 (measured on GB300: 2^15 for 2^20 values, 2^18
// for 2^26; more chunks cost more jumps, longer ones a longer run), scaled
// by mexp / 11213 (a jump's correlation grows with mexp^2, so the best
// length grows with mexp).

int64_t singleChunk(size_t n, int mexp) {
    const double t = 32.0 * (mexp / 11213.0) * std::sqrt((double)n);
    int64_t c = 1;
    while ((double)c * 1.4142135623730951 < t) c <<= 1;
    return c;
}

int waitSlot(SingleFill &F, int i) {
    if (F.done[i])
        CK(cudaEventSynchronize(F.done[i]), "wait for an earlier fill");
    else
        CK(cudaEventCreateWithFlags(&F.done[i], cudaEventDisableTiming), "cudaEventCreate");
    return MTGP_OK;
}

template <class T, class Obj>
int fillSingle(Obj *h, int kind, void *out, size_t n, void *s);

// The same fill as a one-item split plan whose chunks start with in-kernel
// jumps, one CTA per jump, on the one-word core (tuning knob jump_parts =
// -1; about two chunks per SM).
template <class T, class Obj>
int fillSplitPlan(Obj *h, int kind, void *out, size_t n, void *s, int sms) {
    Pool<T> &P = h->pool;
    SingleFill &F = h->fill;
    const int i = F.next;
    int rc = waitSlot(F, i);
    if (rc) return rc;
    mtgp_work_item_t it{};
    it.stream = 0;
    it.kind = kind;
    it.count = n;
    int64_t chunk = P.tune.split_chunk;
    if (chunk == 0) {
        chunk = 1 << 17;
        while ((uint64_t)chunk * 2 * (uint64_t)sms < n) chunk <<= 1;
    }
    rc = makePlan(P, &it, 1, &F.slot[i].plan, 1, chunk);
    if (!rc) rc = launchPlan<T>(F.slot[i].plan, out, s);
    if (rc) return rc;
    CK(cudaEventRecord(F.done[i], S(s)), "record fill");
    F.next ^= 1;
    return MTGP_OK;
}

template <class T, class Obj>
int fillSingle(Obj *h, int kind, void *out, size_t n, void *s) {
    using W = typename T::W;
    Pool<T> &P = h->pool;
    if (n < kSplitFillMin || !T::splits(P.sh.mexp)) return P.fillAll(kind, out, n, s);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(S(s), &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return P.fillAll(kind, out, n, s);
    int rc = P.checkKind(kind);
    if (!rc) rc = P.checkOut(out, n);
    if (rc) return rc;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (P.tune.jump_parts < 0) return fillSplitPlan<T>(h, kind, out, n, s, sms);
    int64_t chunk = P.tune.single_chunk > 0 ? P.tune.single_chunk : singleChunk(n, P.sh.mexp);
    if ((n + chunk - 1) / chunk > (uint64_t)kMaxFillChunks)
        chunk = (int64_t)((n + kMaxFillChunks - 1) / kMaxFillChunks);
    const int nch = (int)((n + chunk - 1) / chunk);
    if (nch < 2) return P.fillAll(kind, out, n, s);
    SingleFill &F = h->fill;
    const int i = F.next;
    SingleFill::Slot &L = F.slot[i];
    rc = waitSlot(F, i);
    if (rc) return rc;

    // chunk-start polynomials X^(c * chunk), c = 1 .. nch - 1
    const int pw = P.polyWords();
    if (F.poly_chunk != chunk || F.npolys < nch - 1) {
        for (int q = 0; q < 2; q++)  // earlier fills may still read them
            if (F.done[q]) CK(cudaEventSynchronize(F.done[q]), "wait for an earlier fill");
        const size_t words = (size_t)(nch - 1) * (size_t)pw;
        F.poly_chunk = 0;
        F.npolys = 0;
        if (words > F.cap_polys) {
            cudaFree(F.d_polys);
            F.d_polys = nullptr;
            F.cap_polys = 0;
            CK(devMalloc(&F.d_polys, sizeof(uint32_t) * words), "devMalloc(chunk polynomials)");
            F.cap_polys = words;
        }
        std::vector<uint64_t> steps((size_t)nch - 1);
        for (int c = 1; c < nch; c++) steps[(size_t)c - 1] = (uint64_t)c * (uint64_t)chunk;
        rc = P.gpuPolys(P.hpidx[0], steps.data(), nch - 1, F.d_polys, s);
        if (rc) return rc;
        // later fills may be issued on other streams
        CK(cudaStreamSynchronize(S(s)), "chunk polynomials");
        F.poly_chunk = chunk;
        F.npolys = nch - 1;
    }

    // windows, and descriptors (rebuilt only when the fill's shape changes)
    const size_t stride = (size_t)P.stride;
    const size_t win_bytes = sizeof(W) * stride * (size_t)nch;
    if (win_bytes > L.cap_win) {
        cudaFree(L.d_win);
        L.d_win = nullptr;
        L.cap_win = 0;
        CK(devMalloc(&L.d_win, win_bytes), "devMalloc(chunk windows)");
        L.cap_win = win_bytes;
    }
    if (!L.d_counter) CK(devMalloc(&L.d_counter, sizeof(unsigned)), "devMalloc(counter)");
    W *win = static_cast<W *>(L.d_win);
    const int tchunks = T::jumpChunks(P.sh.mexp, pw);
    const int parts = jumpParts(P.tune, tchunks);
    const int nparts = (nch - 1) * parts;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t off_items = al(sizeof(BatchTask) * (size_t)nch);
    const size_t off_parts = off_items + al(sizeof(BatchItem) * (size_t)nch);
    const size_t bytes = off_parts + sizeof(JumpPart) * (size_t)nparts;
    if (L.n != n || L.kind != kind || L.chunk != chunk || L.parts != parts || L.win != L.d_win ||
        L.polys != F.d_polys) {
        L.n = 0;
        if (bytes > L.cap_desc) {
            cudaFreeHost(L.h_desc);
            cudaFree(L.d_desc);
            L.h_desc = L.d_desc = nullptr;
            L.cap_desc = 0;
            CK(hostAlloc(&L.h_desc, bytes), "cudaMallocHost(fill descriptors)");
            CK(devMalloc(&L.d_desc, bytes), "devMalloc(fill descriptors)");
            L.cap_desc = bytes;
        }
        BatchTask *t = reinterpret_cast<BatchTask *>(L.h_desc);
        BatchItem *it = reinterpret_cast<BatchItem *>(L.h_desc + off_items);
        JumpPart *jp = reinterpret_cast<JumpPart *>(L.h_desc + off_parts);
        for (int c = 0; c < nch; c++) {
            t[c] = BatchTask{};
            t[c].stream = c;
            t[c].first = c;
            t[c].nitems = 1;
            t[c].pidx = P.hpidx[0];
            t[c].j0 = t[c].j1 = -1;
            t[c].wb = c == nch - 1 ? kWbStream : kWbNone;
            it[c] = BatchItem{};
            it[c].out_off = (uint64_t)c * (uint64_t)chunk * sizeof(W);
            it[c].count = c == nch - 1 ? n - (uint64_t)c * (uint64_t)chunk : (uint64_t)chunk;
            it[c].kind = kind;
        }
        for (int c = 1; c < nch; c++)
            for (int q = 0; q < parts; q++) {
                JumpPart &d = jp[(size_t)(c - 1) * parts + q];
                d = JumpPart{};
                d.src = 0;
                d.poly = c - 1;
                d.dst = c;
                d.pidx = P.hpidx[0];
                d.ch0 = (int16_t)partChunk(q, tchunks, parts);
                d.ch1 = (int16_t)partChunk(q + 1, tchunks, parts);
            }
        CK(cudaMemcpyAsync(L.d_desc, L.h_desc, bytes, cudaMemcpyHostToDevice, S(s)),
           "upload fill descriptors");
        L.n = n;
        L.kind = kind;
        L.chunk = chunk;
        L.parts = parts;
        L.win = L.d_win;
        L.polys = F.d_polys;
    }

    CK(T::windows(P.d_states, win, P.size, (int)stride, nch, S(s)), "chunk windows");
    CK(T::parts(P.sh.mexp, P.d_params, win, F.d_polys, pw, win, (int)stride,
                reinterpret_cast<const JumpPart *>(L.d_desc + off_parts), nparts, S(s)),
       "chunk-start jumps");
    BatchLaunch b{};
    b.mexp = P.sh.mexp;
    b.mode = kind;
    b.grid = std::min(nch, T::resident(P.sh.mexp, false, 2));
    b.core = 2;
    b.split = false;
    b.nwords = pw;
    b.tasks = reinterpret_cast<const BatchTask *>(L.d_desc);
    b.ntasks = nch;
    b.items = reinterpret_cast<const BatchItem *>(L.d_desc + off_items);
    b.out = out;
    b.counter = L.d_counter;
    CK(T::batch(b, P.d_params, win, S(s)), "chunks");
    CK(cudaMemcpyAsync(P.d_states, win + (size_t)(nch - 1) * stride, sizeof(W) * (size_t)P.size,
                       cudaMemcpyDeviceToDevice, S(s)),
       "window after the last chunk");
    CK(cudaEventRecord(F.done[i], S(s)), "record fill");
    F.next ^= 1;
    return MTGP_OK;
}

// Advance one generator by n steps: generated (and discarded) below
// kSkipJumpMin steps, a GF(2) jump by X^n mod chi above (the polynomial made
// on the GPU; a few launches instead of n steps).
constexpr uint64_t kSkipJumpMin = uint64_t(1) << 22;

template <class T>
int skipSingle(Pool<T> &P, uint64_t n, void *s) {
    if (n < kSkipJumpMin) return P.fillOne(0, -1, nullptr, n, s);
    return P.jumpGpu(0, n, s);
}

template <class Obj>
void freeSingle(Obj *h) {
    cudaDeviceSynchronize();
    SingleFill &F = h->fill;
    for (int i = 0; i < 2; i++) {
        SingleFill::Slot &L = F.slot[i];
        delete L.plan;
        cudaFree(L.d_win);
        cudaFree(L.d_desc);
        cudaFreeHost(L.h_desc);
        cudaFree(L.d_counter);
        if (F.done[i]) cudaEventDestroy(F.done[i]);
    }
    cudaFree(F.d_polys);
    delete h;
}

// A single generator from an integer seed, seeded on the device.
template <class T, class Obj>
int initSeeded(Obj **out, const typename T::HP *para, typename T::W seed) {
    int rc = newObj(out);
    if (rc) return rc;
    rc = (*out)->pool.init(para, 1, nullptr, 1);
    if (!rc) rc = (*out)->pool.seedAll(&seed);
    if (rc) {
        delete *out;
        *out = nullptr;
    }
    return rc;
}

// A single generator from a key schedule (init_by_array / init_by_str),
// seeded on the device.
template <class T, class Obj>
int initKeyed(Obj **out, const typename T::HP *para, const typename T::W *keys, int len) {
    int rc = newObj(out);
    if (rc) return rc;
    const uint64_t koff[2] = {0, (uint64_t)len};
    rc = (*out)->pool.init(para, 1, nullptr, 1);
    if (!rc) rc = (*out)->pool.seedKeys(keys, koff);
    if (rc) {
        delete *out;
        *out = nullptr;
    }
    return rc;
}

template <class T>
std::vector<typename T::W> strKeys(const char *str) {
    std::vector<typename T::W> k(std::strlen(str));
    for (size_t j = 0; j < k.size(); j++) k[j] = T::strKey(str[j]);
    return k;
}

template <class T, class Obj>
int importSingle(Obj *h, const typename T::Fast *src) {
    using W = typename T::W;
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    if (!src || !src->status) return setErr(MTGP_ERR_INVALID, "source has no status");
    Shape sh;
    int rc = checkParams<T>(src->params, &sh);
    if (rc) return rc;
    if (sh.mexp != h->pool.sh.mexp)
        return setErr(MTGP_ERR_INVALID, "source exponent %d differs from handle's %d", sh.mexp,
                      h->pool.sh.mexp);
    const int size = h->pool.size;
    int ls = src->status->large_size, idx = src->status->idx;
    if (src->status->size != size || ls <= size || (ls & (ls - 1)))
        return setErr(MTGP_ERR_INVALID, "source status has unexpected sizes");
    std::vector<W> win(size);
    for (int k = 0; k < size; k++) win[k] = src->status->array[(idx - size + 1 + k + ls) & (ls - 1)];
    typename T::DP dp;
    toDev(src->params, &dp);
    CK(cudaDeviceSynchronize(), "synchronize");
    CK(cudaMemcpy(h->pool.d_params, &dp, sizeof dp, cudaMemcpyHostToDevice), "upload params");
    h->pool.hparams[0] = src->params;
    h->pool.chideg[0] = -1;
    return h->pool.setWindows(win.data(), win.size());
}

}  // namespace

extern "C" {

// ---- single generator, 32-bit -------------------------------------------
int mtgp32_gpu_init(mtgp32_gpu_t **out, const mtgp32_params_fast_t *para, uint32_t seed) {
    if (!para) return setErr(MTGP_ERR_INVALID, "null parameter set");
    Shape sh;
    int rc = checkParams<T32>(*para, &sh);
    if (rc) return rc;
    return initSeeded<T32>(out, para, seed);
}
int mtgp32_gpu_init_by_array(mtgp32_gpu_t **out, const mtgp32_params_fast_t *para,
                             const uint32_t *array, int length) {
    if (!para || length < 0 || (length > 0 && !array))
        return setErr(MTGP_ERR_INVALID, "bad seed array");
    Shape sh;
    int rc = checkParams<T32>(*para, &sh);
    if (rc) return rc;
    return initKeyed<T32>(out, para, array, length);
}
int mtgp32_gpu_init_by_str(mtgp32_gpu_t **out, const mtgp32_params_fast_t *para, const char *str) {
    if (!para || !str) return setErr(MTGP_ERR_INVALID, "bad seed string");
    Shape sh;
    int rc = checkParams<T32>(*para, &sh);
    if (rc) return rc;
    const std::vector<uint32_t> k = strKeys<T32>(str);
    return initKeyed<T32>(out, para, k.data(), (int)k.size());
}
void mtgp32_gpu_free(mtgp32_gpu_t *h) {
    if (!h) return;
    freeSingle(h);
}
int mtgp32_gpu_fill(mtgp32_gpu_t *h, int kind, void *out, size_t n, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return fillSingle<T32>(h, kind, out, n, s);
}
int mtgp32_gpu_fill_uint32(mtgp32_gpu_t *h, uint32_t *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 0, o, n, s); }
int mtgp32_gpu_fill_close1_open2(mtgp32_gpu_t *h, float *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 1, o, n, s); }
int mtgp32_gpu_fill_close_open(mtgp32_gpu_t *h, float *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 2, o, n, s); }
int mtgp32_gpu_fill_open_close(mtgp32_gpu_t *h, float *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 3, o, n, s); }
int mtgp32_gpu_fill_open_open(mtgp32_gpu_t *h, float *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 4, o, n, s); }
int mtgp32_gpu_skip(mtgp32_gpu_t *h, uint64_t n, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return skipSingle(h->pool, n, s);
}
int mtgp32_gpu_fast_jump(mtgp32_gpu_t *h, const char *js, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.fastJump(0, js, s);
}
int mtgp32_gpu_jump_array(mtgp32_gpu_t *h, const uint32_t *p, int nw, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.jumpArray(0, p, nw, s);
}
int mtgp32_gpu_jump_steps(mtgp32_gpu_t *h, uint64_t lo, uint64_t hi, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.jumpSteps(0, lo, hi, s);
}
int mtgp32_gpu_export(mtgp32_gpu_t *h, mtgp32_fast_t *dst) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.exportTo(0, dst);
}
int mtgp32_gpu_import(mtgp32_gpu_t *h, const mtgp32_fast_t *src) { return importSingle<T32>(h, src); }
int mtgp32_gpu_get_window_host(mtgp32_gpu_t *h, uint32_t *w, int size) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.getWindows(w, size < 0 ? 0 : (size_t)size);
}
int mtgp32_gpu_set_window_host(mtgp32_gpu_t *h, const uint32_t *w, int size) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.setWindows(w, size < 0 ? 0 : (size_t)size);
}

// ---- single generator, 64-bit -------------------------------------------
int mtgp64_gpu_init(mtgp64_gpu_t **out, const mtgp64_params_fast_t *para, uint64_t seed) {
    if (!para) return setErr(MTGP_ERR_INVALID, "null parameter set");
    Shape sh;
    int rc = checkParams<T64>(*para, &sh);
    if (rc) return rc;
    return initSeeded<T64>(out, para, seed);
}
int mtgp64_gpu_init_by_array(mtgp64_gpu_t **out, const mtgp64_params_fast_t *para,
                             const uint64_t *array, int length) {
    if (!para || length < 0 || (length > 0 && !array))
        return setErr(MTGP_ERR_INVALID, "bad seed array");
    Shape sh;
    int rc = checkParams<T64>(*para, &sh);
    if (rc) return rc;
    return initKeyed<T64>(out, para, array, length);
}
int mtgp64_gpu_init_by_str(mtgp64_gpu_t **out, const mtgp64_params_fast_t *para, const char *str) {
    if (!para || !str) return setErr(MTGP_ERR_INVALID, "bad seed string");
    Shape sh;
    int rc = checkParams<T64>(*para, &sh);
    if (rc) return rc;
    const std::vector<uint64_t> k = strKeys<T64>(str);
    return initKeyed<T64>(out, para, k.data(), (int)k.size());
}
void mtgp64_gpu_free(mtgp64_gpu_t *h) {
    if (!h) return;
    freeSingle(h);
}
int mtgp64_gpu_fill(mtgp64_gpu_t *h, int kind, void *out, size_t n, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return fillSingle<T64>(h, kind, out, n, s);
}
int mtgp64_gpu_fill_uint64(mtgp64_gpu_t *h, uint64_t *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 0, o, n, s); }
int mtgp64_gpu_fill_close1_open2(mtgp64_gpu_t *h, double *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 1, o, n, s); }
int mtgp64_gpu_fill_close_open(mtgp64_gpu_t *h, double *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 2, o, n, s); }
int mtgp64_gpu_fill_open_close(mtgp64_gpu_t *h, double *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 3, o, n, s); }
int mtgp64_gpu_fill_open_open(mtgp64_gpu_t *h, double *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 4, o, n, s); }
int mtgp64_gpu_skip(mtgp64_gpu_t *h, uint64_t n, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return skipSingle(h->pool, n, s);
}
int mtgp64_gpu_fast_jump(mtgp64_gpu_t *h, const char *js, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.fastJump(0, js, s);
}
int mtgp64_gpu_jump_array(mtgp64_gpu_t *h, const uint32_t *p, int nw, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.jumpArray(0, p, nw, s);
}
int mtgp64_gpu_jump_steps(mtgp64_gpu_t *h, uint64_t lo, uint64_t hi, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.jumpSteps(0, lo, hi, s);
}
int mtgp64_gpu_export(mtgp64_gpu_t *h, mtgp64_fast_t *dst) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.exportTo(0, dst);
}
int mtgp64_gpu_import(mtgp64_gpu_t *h, const mtgp64_fast_t *src) { return importSingle<T64>(h, src); }
int mtgp64_gpu_get_window_host(mtgp64_gpu_t *h, uint64_t *w, int size) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.getWindows(w, size < 0 ? 0 : (size_t)size);
}
int mtgp64_gpu_set_window_host(mtgp64_gpu_t *h, const uint64_t *w, int size) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.setWindows(w, size < 0 ? 0 : (size_t)size);
}

int mtgp32_gpu_gen_set_tuning(mtgp32_gpu_t *h, const char *key, int64_t value) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null generator");
    return applyTuning(h->pool.tune, key, value);
}
int mtgp64_gpu_gen_set_tuning(mtgp64_gpu_t *h, const char *key, int64_t value) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null generator");
    return applyTuning(h->pool.tune, key, value);
}

}  // extern "C"
