// The C library's rand() stream and std::random_shuffle, replayed on the device: the
// shuffled relabellings of vertex_ordering/A-order (relabel-naive.cpp:145-147 and
// relabel4lpOut.cpp:105-107 shuffle blocks of a dealt degree list; relabel-random.cpp:81
// shuffles all ids).  The programs never call srand, so their rand() is the C library's
// generator in its seed-1 state, and the output bytes depend on the exact stream.
//
// rand(): glibc's default generator (TYPE_3, an additive lagged-Fibonacci generator of
// degree 31 and separation 3), as published in P. Selinger, "The GLIBC pseudo-random number
// generator" (2007):
//   r[0] = seed = 1;  r[i] = 16807 r[i-1] mod (2^31 - 1) for i = 1..30;
//   r[i] = r[i-31] for i = 31..33;  r[i] = r[i-3] + r[i-31] mod 2^32 for i >= 34;
//   call k (k = 0, 1, ...) returns r[k + 344] >> 1.
// With a[j] = r[j + 3] the recurrence is a[j] = a[j-3] + a[j-31] for j >= 31, linear over
// Z/2^32, so a[j] = sum_i c_i a[i] (i < 31) where sum_i c_i x^i = x^j mod (x^31 - x^28 - 1).
// Each thread raises x to the start of its own stretch of the stream, takes the 31 values
// before it from the seed values, and runs the recurrence from there.
//
// std::random_shuffle(first, last) of libstdc++: for i = 1 .. len-1, swap(a[i], a[j]) with
// j = rand() % (i + 1).  A block shuffle is that loop, one thread per block.  The shuffle of
// all n ids is replayed in parallel: with H[i] = the j of step i, position i holds its own
// id until step i, so step i moves id i to H[i] and the previous holder of H[i] to i.  The
// holder of position q just before step t (q < t) is therefore the largest k < t with
// H[k] = q (k = q when H[q] = q), or, when there is none, the holder of H[q] just before
// step q (q = 0: id 0).  Every position follows that chain down to its answer; the chain
// visits strictly decreasing positions, about ln n of them.  The steps are grouped by
// their target (a radix sort of (H[k], k)) so each visit searches a short sorted run.
#include "internal.cuh"

namespace atc {
namespace {

constexpr int kDeg = 31;            // degree of the generator's recurrence
constexpr int kStretch = 2048;      // stream values per thread
constexpr int64_t kSkip = 341;      // call k returns a[k + kSkip] >> 1

// the 31 seed values a[0..30] = r[3..33] of seed 1
__device__ void seed_values(uint32_t* a) {
  uint32_t r[kDeg];
  int64_t x = 1;
  r[0] = 1;
  for (int i = 1; i < kDeg; ++i) {
    x = (16807 * x) % 2147483647;
    r[i] = (uint32_t)x;
  }
  for (int i = 0; i < 28; ++i) a[i] = r[i + 3];     // r[3..30]
  for (int i = 28; i < kDeg; ++i) a[i] = r[i - 28];  // r[31..33] = r[0..2]
}

// p <- p * q mod (x^31 - x^28 - 1), coefficients mod 2^32
__device__ void poly_mulmod(uint32_t* p, const uint32_t* q) {
  uint32_t t[2 * kDeg - 1];
  for (int i = 0; i < 2 * kDeg - 1; ++i) t[i] = 0;
  for (int i = 0; i < kDeg; ++i) {
    const uint32_t pi = p[i];
    if (pi == 0) continue;
    for (int j = 0; j < kDeg; ++j) t[i + j] += pi * q[j];
  }
  for (int d = 2 * kDeg - 2; d >= kDeg; --d) {  // x^d = x^(d-31) (x^28 + 1)
    t[d - 3] += t[d];
    t[d - kDeg] += t[d];
  }
  for (int i = 0; i < kDeg; ++i) p[i] = t[i];
}

// out[k] = the value of rand() call k, k < count
__global__ void rand_stream_kernel(uint32_t* out, int64_t count) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t k0 = t * kStretch;
  if (k0 >= count) return;
  uint32_t a0[kDeg], c[kDeg], x[kDeg], ring[kDeg];
  seed_values(a0);
  // c = x^(j0 - 31) mod f, j0 = k0 + kSkip the first a-index this thread writes
  for (int i = 0; i < kDeg; ++i) c[i] = 0, x[i] = 0;
  c[0] = 1;
  x[1] = 1;
  for (uint64_t e = (uint64_t)(k0 + kSkip - kDeg); e; e >>= 1) {
    if (e & 1) poly_mulmod(c, x);
    if (e > 1) poly_mulmod(x, x);
  }
  // ring = a[j0-31 .. j0-1]: coefficients of x^(j0-31+i) = c * x^i
  for (int i = 0; i < kDeg; ++i) {
    uint32_t v = 0;
    for (int j = 0; j < kDeg; ++j) v += c[j] * a0[j];
    ring[i] = v;
    const uint32_t top = c[kDeg - 1];  // c <- c * x: x^31 = x^28 + 1
    for (int j = kDeg - 1; j > 0; --j) c[j] = c[j - 1];
    c[0] = top;
    c[28] += top;
  }
  const int64_t k1 = min(count, k0 + kStretch);
  int h = 0;  // ring[h] = a[j-31], ring[(h+28) % 31] = a[j-3]
  for (int64_t k = k0; k < k1; ++k) {
    const int h3 = h + 28 < kDeg ? h + 28 : h + 28 - kDeg;
    const uint32_t v = ring[h] + ring[h3];
    ring[h] = v;
    h = h + 1 < kDeg ? h + 1 : 0;
    out[k] = v >> 1;
  }
}

// random_shuffle of every block [b*width, (b+1)*width), b < nblocks, in block order: block
// b takes calls [b*(width-1), (b+1)*(width-1)) of the stream.
__global__ void block_shuffle_kernel(int32_t* a, int64_t nblocks, int width, const uint32_t* rnd) {
  int32_t v[kMaxShuffleWidth];
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nblocks; b += (int64_t)gridDim.x * blockDim.x) {
    int32_t* p = a + b * width;
    const uint32_t* r = rnd + b * (width - 1);
    for (int i = 0; i < width; ++i) v[i] = p[i];
    for (int i = 1; i < width; ++i) {
      const int j = (int)(r[i - 1] % (uint32_t)(i + 1));
      const int32_t s = v[i];
      v[i] = v[j];
      v[j] = s;
    }
    for (int i = 0; i < width; ++i) p[i] = v[i];
  }
}

// H[i] = the swap partner of step i (i = 1..n-1), as the key (H[i] << 32 | i)
__global__ void step_keys_kernel(const uint32_t* rnd, int64_t n, uint64_t* keys, int32_t* target) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + 1; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t h = (uint32_t)((uint64_t)rnd[i - 1] % (uint64_t)(i + 1));
    keys[i - 1] = ((uint64_t)h << 32) | (uint64_t)i;
    target[i] = (int32_t)h;
  }
}

// start[q] = first sorted step with target >= q (q = 0..n)
__global__ void step_starts_kernel(const uint64_t* keys, int64_t nsteps, int64_t n, int64_t* start) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q <= n; q += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = nsteps;
    const uint64_t key = (uint64_t)q << 32;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] < key) lo = mid + 1; else hi = mid;
    }
    start[q] = lo;
  }
}

// out[p] = the id at position p after the whole shuffle of 0..n-1
__global__ void shuffle_holder_kernel(const uint64_t* keys, const int64_t* start, const int32_t* target, int64_t n,
                                      int32_t* out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = p, t = n;
    int32_t id = 0;
    for (;;) {  // q strictly decreases: at most p + 1 rounds
      // the last step k < t of the run of target q (runs are sorted by k)
      int64_t lo = start[q], hi = start[q + 1];
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)(keys[mid] & 0xffffffffull) < t) lo = mid + 1; else hi = mid;
      }
      if (lo > start[q]) {
        id = (int32_t)(keys[lo - 1] & 0xffffffffull);
        break;
      }
      if (q == 0) {
        id = 0;
        break;
      }
      t = q;
      q = target[q];
    }
    out[p] = id;
  }
}

__global__ void iota_kernel(int32_t* a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = (int32_t)i;
}

}  // namespace

atc_status rand_stream(uint32_t* out, int64_t count, cudaStream_t s) {
  if (count <= 0) return ATC_OK;
  const int64_t threads = (count + kStretch - 1) / kStretch;
  rand_stream_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(out, count);
  ATC_CK(cudaGetLastError());
  return ATC_OK;
}

atc_status shuffle_blocks(int32_t* a, int64_t nblocks, int width, cudaStream_t s) {
  ATC_CHECK_ARG(width >= 1 && width <= kMaxShuffleWidth, "shuffle block width out of range");
  if (nblocks <= 0 || width < 2) return ATC_OK;
  DevBuf<uint32_t> rnd;
  ATC_TRY(rnd.alloc(nblocks * (width - 1), s));
  ATC_TRY(rand_stream(rnd.p, nblocks * (width - 1), s));
  block_shuffle_kernel<<<grid_for(nblocks, 128), 128, 0, s>>>(a, nblocks, width, rnd.p);
  ATC_CK(cudaGetLastError());
  return ATC_OK;
}

atc_status shuffle_ids(int32_t* out, int64_t n, cudaStream_t s) {
  if (n <= 0) return ATC_OK;
  ATC_CHECK_ARG(n <= (int64_t)INT32_MAX, "too many ids to shuffle");
  if (n == 1) {
    iota_kernel<<<1, 32, 0, s>>>(out, 1);
    ATC_CK(cudaGetLastError());
    return ATC_OK;
  }
  const int64_t nsteps = n - 1;
  DevBuf<uint32_t> rnd;
  DevBuf<uint64_t> ka, kb;
  DevBuf<int32_t> target;
  DevBuf<int64_t> start;
  ATC_TRY(rnd.alloc(nsteps, s));
  ATC_TRY(ka.alloc(nsteps, s));
  ATC_TRY(kb.alloc(nsteps, s));
  ATC_TRY(target.alloc(n, s));
  ATC_TRY(start.alloc(n + 1, s));
  ATC_TRY(rand_stream(rnd.p, nsteps, s));
  step_keys_kernel<<<grid_for(nsteps, 256), 256, 0, s>>>(rnd.p, n, ka.p, target.p);
  ATC_CK(cudaGetLastError());
  rnd.release();
  const int bits = id_bits(n);
  uint64_t* a = ka.p;
  uint64_t* b = kb.p;
  ATC_TRY(sort_keys_u64(a, b, nsteps, 0, 32 + bits, s));
  step_starts_kernel<<<grid_for(n + 1, 256), 256, 0, s>>>(a, nsteps, n, start.p);
  ATC_CK(cudaGetLastError());
  shuffle_holder_kernel<<<grid_for(n, 256), 256, 0, s>>>(a, start.p, target.p, n, out);
  ATC_CK(cudaGetLastError());
  return ATC_OK;
}

}  // namespace atc
