// Monolith-12 over Goldilocks and its Merkle trees (the goldilocks-cuda-rs default Merkle hash,
// goldilocks-cuda-rs/Cargo.toml:22-24): the reference ABI monolith_* (src/ffi.rs:565-582,
// wrapper.cu:1889-2011), semantics of goldilocks-cuda-rs/src/cpu_monolith.rs:13-226.
//   permutation: concrete(0), then 6 x (bars on limbs 0..3, bricks, concrete(r));
//   concrete:    out[r] = sum_c MDS[r][c] s[c] + RC[round][r] with the circulant MDS whose first
//                row is (7, 23, 8, 26, 13, 10, 9, 7, 6, 22, 21, 8), reduced to canonical form
//                (the bars read the limbs' bits);
//   bricks:      s[i] += s[i-1]^2 for i = 11 .. 1, every square from the state before the step.
// Leaves: gl H(cw[2i], cw[2i+1], 0, ...), ext2 H(cw[4i..4i+3], 0, ...); compress H(l || r);
// digests are the first 4 words.  Tree layout as the Poseidon2 trees (leaves first, 4 words per
// node).  One permutation per thread.
#include "../../include/goldilocks_cuda_wrapper.h"
#include "common.cuh"
#include "gl.cuh"

namespace gb {

#define GB_MO_RC                                                                                          \
    {{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},                                                               \
     {13596126580325903823ull, 5676126986831820406ull, 11349149288412960427ull, 3368797843020733411ull,   \
      16240671731749717664ull, 9273190757374900239ull, 14446552112110239438ull, 4033077683985131644ull,   \
      4291229347329361293ull, 13231607645683636062ull, 1383651072186713277ull, 8898815177417587567ull},   \
     {2383619671172821638ull, 6065528368924797662ull, 16737578966352303081ull, 2661700069680749654ull,    \
      7414030722730336790ull, 18124970299993404776ull, 9169923000283400738ull, 15832813151034110977ull,   \
      16245117847613094506ull, 11056181639108379773ull, 10546400734398052938ull, 8443860941261719174ull}, \
     {15799082741422909885ull, 13421235861052008152ull, 15448208253823605561ull, 2540286744040770964ull,  \
      2895626806801935918ull, 8644593510196221619ull, 17722491003064835823ull, 5166255496419771636ull,    \
      1015740739405252346ull, 4400043467547597488ull, 5176473243271652644ull, 4517904634837939508ull},    \
     {18341030605319882173ull, 13366339881666916534ull, 6291492342503367536ull, 10004214885638819819ull,  \
      4748655089269860551ull, 1520762444865670308ull, 8393589389936386108ull, 11025183333304586284ull,    \
      5993305003203422738ull, 458912836931247573ull, 5947003897778655410ull, 17184667486285295106ull},    \
     {15710528677110011358ull, 8929476121507374707ull, 2351989866172789037ull, 11264145846854799752ull,   \
      14924075362538455764ull, 10107004551857451916ull, 18325221206052792232ull, 16751515052585522105ull, \
      15305034267720085905ull, 15639149412312342017ull, 14624541102106656564ull, 3542311898554959098ull}, \
     {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}}

__device__ __forceinline__ u64 mo_rc(int r, int i) {
    constexpr u64 t[7][12] = GB_MO_RC;
    return t[r][i];
}
__device__ __forceinline__ u32 mo_c(int k) {
    constexpr u32 t[12] = {7, 23, 8, 26, 13, 10, 9, 7, 6, 22, 21, 8};
    return t[k];
}

__device__ __forceinline__ u64 mo_bar(u64 x) {
    u64 l1 = ((~x & 0x8080808080808080ull) >> 7) | ((~x & 0x7F7F7F7F7F7F7F7Full) << 1);
    u64 l2 = ((x & 0xC0C0C0C0C0C0C0C0ull) >> 6) | ((x & 0x3F3F3F3F3F3F3F3Full) << 2);
    u64 l3 = ((x & 0xE0E0E0E0E0E0E0E0ull) >> 5) | ((x & 0x1F1F1F1F1F1F1F1Full) << 3);
    u64 t = x ^ (l1 & l2 & l3);
    return ((t & 0x8080808080808080ull) >> 7) | ((t & 0x7F7F7F7F7F7F7F7Full) << 1);
}

// concrete layer: each row summed as (sum of c * low halves) + 2^32 (sum of c * high halves) +
// RC in 128 bits (every coefficient is below 2^5, twelve terms), reduced once, canonical
__device__ __forceinline__ void mo_concrete(u64* s, int round) {
    u32 lo[12], hi[12];
#pragma unroll
    for (int i = 0; i < 12; i++) {
        lo[i] = (u32)s[i];
        hi[i] = (u32)(s[i] >> 32);
    }
#pragma unroll
    for (int r = 0; r < 12; r++) {
        u64 a = 0, b = 0;
#pragma unroll
        for (int c = 0; c < 12; c++) {
            const u32 m = mo_c((c - r + 12) % 12);
            a += (u64)lo[c] * m;
            b += (u64)hi[c] * m;
        }
        // a + 2^32 b + rc, b < 2^42
        u64 x = a + (b << 32);
        u64 h = (b >> 32) + (x < a ? 1 : 0);
        u64 rc = mo_rc(round, r);
        u64 y = x + rc;
        h += (y < x) ? 1 : 0;
        s[r] = gl_canon(gl_reduce(y, h));
    }
}

__device__ __forceinline__ void mo_permute(u64* s) {
#pragma unroll
    for (int i = 0; i < 12; i++) s[i] = gl_canon(s[i]);
    mo_concrete(s, 0);
#pragma unroll 1
    for (int r = 1; r <= 6; r++) {
#pragma unroll
        for (int i = 0; i < 4; i++) s[i] = mo_bar(s[i]);
        u64 sq[11];
#pragma unroll
        for (int i = 0; i < 11; i++) sq[i] = gl_sqr(s[i]);
#pragma unroll
        for (int i = 1; i < 12; i++) s[i] = gl_canon(gl_add(s[i], sq[i - 1]));
        mo_concrete(s, r);
    }
}

// width words per leaf (2: base pair, 4: Ext2 pair)
__global__ void mo_leaves_kernel(const u64* __restrict__ cw, u64* __restrict__ tree, size_t leaves, int width) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= leaves) return;
    u64 s[12];
#pragma unroll
    for (int k = 0; k < 12; k++) s[k] = 0;
    for (int k = 0; k < width; k++) s[k] = cw[(size_t)width * i + k];
    mo_permute(s);
#pragma unroll
    for (int k = 0; k < 4; k++) tree[4 * i + k] = s[k];
}

__global__ void mo_level_kernel(const u64* __restrict__ in, u64* __restrict__ out, size_t parents) {
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= parents) return;
    u64 s[12];
#pragma unroll
    for (int k = 0; k < 8; k++) s[k] = in[8 * j + k];
#pragma unroll
    for (int k = 8; k < 12; k++) s[k] = 0;
    mo_permute(s);
#pragma unroll
    for (int k = 0; k < 4; k++) out[4 * j + k] = s[k];
}

__global__ void mo_permute_kernel(u64* __restrict__ s) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        u64 t[12];
        for (int k = 0; k < 12; k++) t[k] = s[k];
        mo_permute(t);
        for (int k = 0; k < 12; k++) s[k] = t[k];
    }
}

static int mo_tree(const u64* cw, u64* tree, size_t leaves, int width) {
    if (!cw || !tree || leaves == 0) return GB_EINVAL;
    cudaStream_t s = stream();
    mo_leaves_kernel<<<grid_for(leaves, 128), 128, 0, s>>>(cw, tree, leaves, width);
    GB_LAUNCH_CHECK("mo_leaves_kernel");
    size_t off = 0, nodes = leaves;
    while (nodes > 1) {
        size_t parents = nodes / 2;
        mo_level_kernel<<<grid_for(parents, 128), 128, 0, s>>>(tree + 4 * off, tree + 4 * (off + nodes), parents);
        GB_LAUNCH_CHECK("mo_level_kernel");
        off += nodes;
        nodes = parents;
    }
    return sync_stream("monolith_merkle_tree");
}

}  // namespace gb

using namespace gb;

extern "C" {

int monolith_cuda_init(void) { return GB_OK; }

int monolith_merkle_tree_gl_ffi(const uint64_t* d_codeword, uint64_t* d_tree, int num_leaves) {
    if (num_leaves <= 0) return GB_EINVAL;
    return mo_tree(d_codeword, d_tree, (size_t)num_leaves, 2);
}

int monolith_merkle_tree_ext2_ffi(const uint64_t* d_codeword, uint64_t* d_tree, int num_leaves) {
    if (num_leaves <= 0) return GB_EINVAL;
    return mo_tree(d_codeword, d_tree, (size_t)num_leaves, 4);
}

int monolith_permute_test_ffi(const uint64_t* h_input, uint64_t* h_output) {
    if (!h_input || !h_output) return GB_EINVAL;
    cudaStream_t s = stream();
    u64* d = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&d, 12 * 8, s));
    int rc = GB_OK;
    if (cudaMemcpyAsync(d, h_input, 96, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = GB_ECUDA;
    if (!rc) {
        mo_permute_kernel<<<1, 32, 0, s>>>(d);
        rc = check_launch("mo_permute_kernel");
    }
    if (!rc && cudaMemcpyAsync(h_output, d, 96, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = GB_ECUDA;
    cudaFreeAsync(d, s);
    if (!rc) rc = sync_stream("monolith_permute_test_ffi");
    return rc;
}

}  // extern "C"
