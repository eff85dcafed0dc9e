// Background sequences for the e-value filter: a k-let preserving shuffle of every
// sequence, on the device.
//
// The reference makes its background with MEME's `fasta-shuffle-letters -kmer 3`
// (src/SETUP/LOAD_setup.jl:5-14), an external program that is not part of the
// reference.  This is a project-written replacement with the same contract: each
// sequence is replaced by a random sequence with the same length, the same first and
// last (k-1)-mers and exactly the same count of every k-mer.  The method is the
// Euler-path shuffle of Altschul & Erickson (Mol. Biol. Evol. 1985), with the random
// arborescence drawn by Wilson's loop-erased random walk (as in uShuffle, Jiang et al.,
// BMC Bioinformatics 2008): the (k-1)-mers are vertices, the k-mers of the sequence are
// edges; for every vertex but the last one a random "last exit" edge is chosen so that
// the last exits form a tree towards the last vertex, the other exits of each vertex are
// put in random order, and the walk from the first vertex spells the new sequence.
//
// The random numbers are splitmix64 (Steele, Lea & Flood, OOPSLA 2014) on a per-sequence
// counter, so the result depends only on (seed, sequence index) and matches the oracle
// draw for draw.  Symbols: 0..3 = A C G T, 4 = a column with no base (not one-hot).
#include "cdlgb_internal.h"

namespace {

constexpr int kAlpha = 5;
constexpr int kMaxK = 4;
constexpr int kMaxV = 125;                 // kAlpha^(kMaxK - 1)
constexpr long kMaxWalk = 1L << 24;        // bound on the loop-erased walks of one sequence

struct ShArgs {
    const float* S;       // (N, 4L) one-hot
    float* out;           // (N, 4L) shuffled one-hot
    uint8_t* lists;       // scratch (N, L): exits of every vertex, grouped by vertex
    int32_t* err;         // set to 1 when a walk bound is hit
    unsigned long long seed;
    int N, L, k;
};

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Rng {
    unsigned long long s;
    __device__ explicit Rng(unsigned long long seed, int n)
        : s(mix64(seed ^ (0x9E3779B97F4A7C15ull * (unsigned long long)(n + 1)))) {}
    // uniform in [0, m): the high 32 bits scaled by m
    __device__ unsigned below(unsigned m) {
        s += 0x9E3779B97F4A7C15ull;
        const unsigned long long z = mix64(s);
        return (unsigned)(((z >> 32) * (unsigned long long)m) >> 32);
    }
};

__device__ __forceinline__ int symbol_at(const float* x) {
    const float4 v = *reinterpret_cast<const float4*>(x);
    const float c[4] = {v.x, v.y, v.z, v.w};
    int s = 4, ones = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        if (c[a] == 1.f) { ++ones; s = a; }
        else if (c[a] != 0.f) ones = 2;
    }
    return ones == 1 ? s : 4;
}

__device__ __forceinline__ void put_symbol(float* x, int s) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (s == 0) v.x = 1.f; else if (s == 1) v.y = 1.f; else if (s == 2) v.z = 1.f; else if (s == 3) v.w = 1.f;
    *reinterpret_cast<float4*>(x) = v;
}

// Fisher-Yates (Durstenfeld): i from m-1 down to 1, swap a[i] with a[below(i+1)]
__device__ void shuffle_bytes(uint8_t* a, int m, Rng& r) {
    for (int i = m - 1; i >= 1; --i) {
        const int j = (int)r.below((unsigned)(i + 1));
        const uint8_t t = a[i]; a[i] = a[j]; a[j] = t;
    }
}

// one thread per sequence
__global__ void __launch_bounds__(128) k_klet_shuffle(ShArgs A) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= A.N) return;
    const size_t L4 = (size_t)4 * A.L;
    const float* x = A.S + (size_t)n * L4;
    float* y = A.out + (size_t)n * L4;
    uint8_t* lst = A.lists + (size_t)n * A.L;
    Rng rng(A.seed, n);
    const int k = A.k, L = A.L;

    if (k == 1) {
        for (int i = 0; i < L; ++i) lst[i] = (uint8_t)symbol_at(x + 4 * i);
        shuffle_bytes(lst, L, rng);
        for (int i = 0; i < L; ++i) put_symbol(y + 4 * i, lst[i]);
        return;
    }
    const int E = L - k + 1;               // edges (k-mers)
    if (E <= 0) {
        for (int i = 0; i < L; ++i) put_symbol(y + 4 * i, symbol_at(x + 4 * i));
        return;
    }
    int V = 1;
    for (int j = 0; j < k - 1; ++j) V *= kAlpha;
    short deg[kMaxV], off[kMaxV + 1], cur[kMaxV], nxt[kMaxV];
    uint8_t intree[kMaxV];
    for (int v = 0; v < V; ++v) { deg[v] = 0; cur[v] = 0; intree[v] = 0; nxt[v] = 0; }

    // vertex of the first (k-1)-mer, then the exits in sequence order (two passes: the
    // second fills each vertex's exits in the order they occur)
    int v0 = 0;
    for (int j = 0; j < k - 1; ++j) v0 = v0 * kAlpha + symbol_at(x + 4 * j);
    int u = v0;
    for (int i = 0; i < E; ++i) {
        const int w = symbol_at(x + 4 * (i + k - 1));
        ++deg[u];
        u = (u * kAlpha + w) % V;
    }
    const int vend = u;
    off[0] = 0;
    for (int v = 0; v < V; ++v) off[v + 1] = (short)(off[v] + deg[v]);
    u = v0;
    for (int i = 0; i < E; ++i) {
        const int w = symbol_at(x + 4 * (i + k - 1));
        lst[off[u] + cur[u]++] = (uint8_t)w;
        u = (u * kAlpha + w) % V;
    }

    // random arborescence towards vend (Wilson): nxt[v] = index of v's last exit
    intree[vend] = 1;
    long steps = 0;
    for (int v = 0; v < V; ++v) {
        if (deg[v] == 0 || intree[v]) continue;
        u = v;
        while (!intree[u]) {
            if (++steps > kMaxWalk) { atomicExch(A.err, 1); return; }
            nxt[u] = (short)rng.below((unsigned)deg[u]);
            u = (u * kAlpha + lst[off[u] + nxt[u]]) % V;
        }
        u = v;
        while (!intree[u]) {
            intree[u] = 1;
            u = (u * kAlpha + lst[off[u] + nxt[u]]) % V;
        }
    }
    // exits of every vertex in random order, the last exit last
    for (int v = 0; v < V; ++v) {
        const int m = deg[v];
        if (m == 0) continue;
        uint8_t* e = lst + off[v];
        if (v != vend) {
            const uint8_t t = e[nxt[v]]; e[nxt[v]] = e[m - 1]; e[m - 1] = t;
            shuffle_bytes(e, m - 1, rng);
        } else {
            shuffle_bytes(e, m, rng);
        }
        cur[v] = 0;
    }
    // the walk spells the shuffled sequence
    for (int j = 0; j < k - 1; ++j) put_symbol(y + 4 * j, symbol_at(x + 4 * j));
    u = v0;
    for (int i = 0; i < E; ++i) {
        if (cur[u] >= deg[u]) { atomicExch(A.err, 1); return; }   // not reached for an Euler path
        const int w = lst[off[u] + cur[u]++];
        put_symbol(y + 4 * (i + k - 1), w);
        u = (u * kAlpha + w) % V;
    }
}

}  // namespace

int make_background(cdlgb_ctx* c, int k, unsigned long long seed) {
    if (!c->loaded) return cdlgb_seterr(c, CDLGB_ESTATE, "no data loaded");
    if (!c->onehot_exact)
        return cdlgb_seterr(c, CDLGB_ENOTSUP, "make_background: needs 0/1 one-hot data");
    if (k < 1 || k > kMaxK)
        return cdlgb_seterr(c, CDLGB_EINVAL, "make_background: k=%d outside 1..%d", k, kMaxK);
    const int N = c->N, L = c->L4 / 4;
    if (L > 32000) return cdlgb_seterr(c, CDLGB_EINVAL, "make_background: L=%d above 32000", L);
    const size_t n = (size_t)c->L4 * N;
    if (!c->S_bg) ST_TRY(dev_alloc(c, (void**)&c->S_bg, n * 4));
    uint8_t* lists = nullptr;
    int32_t* err = nullptr;
    ST_TRY(dev_alloc(c, (void**)&lists, (size_t)N * L + 16));
    err = reinterpret_cast<int32_t*>(lists + (((size_t)N * L + 3) & ~(size_t)3));
    CU_TRY(c, cudaMemsetAsync(err, 0, 4, c->stream));
    ShArgs a;
    a.S = c->S; a.out = c->S_bg; a.lists = lists; a.err = err; a.seed = seed;
    a.N = N; a.L = L; a.k = k;
    k_klet_shuffle<<<(N + 127) / 128, 128, 0, c->stream>>>(a);
    LAUNCH_CHECK(c, "k_klet_shuffle");
    int32_t herr = 0;
    CU_TRY(c, cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, c->stream));
    dev_free(c, lists);
    CU_TRY(c, cudaStreamSynchronize(c->stream));
    if (herr) {
        c->bg_valid = 0;
        c->use_bg = 0;
        return cdlgb_seterr(c, CDLGB_ETIMEOUT, "make_background: random walk bound reached");
    }
    c->bg_valid = 1;
    return CDLGB_OK;
}
