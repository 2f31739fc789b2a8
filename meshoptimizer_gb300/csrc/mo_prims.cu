// mo_prims.cu - device-wide exclusive scan and stable LSD radix sort.
//
// Both are plain HBM-streaming integer kernels: the scan reads each element twice and
// writes it once (reduce pass + apply pass, with a small recursive scan of tile sums in
// between); each radix pass reads the pairs twice (histogram + scatter) and writes them
// once. Tiles are sized so that a grid of a few thousand blocks covers the 152 SMs.
#include "mo_common.cuh"
#include "mo_grid.cuh"
#include "mo_prims.cuh"
#include "mo_probe.cuh"

#include <algorithm>
#include <atomic>

namespace mogpu
{

namespace
{

__device__ __forceinline__ uint4 loadTile4(const unsigned int* in, size_t n, size_t i, bool aligned)
{
	if (aligned && i + 3 < n)
		return *reinterpret_cast<const uint4*>(in + i);
	uint4 r;
	r.x = i + 0 < n ? in[i + 0] : 0u;
	r.y = i + 1 < n ? in[i + 1] : 0u;
	r.z = i + 2 < n ? in[i + 2] : 0u;
	r.w = i + 3 < n ? in[i + 3] : 0u;
	return r;
}

__global__ void __launch_bounds__(kScanThreads) kScanReduce(const unsigned int* __restrict__ in, size_t n, unsigned int* __restrict__ sums, bool aligned)
{
	__shared__ unsigned int smem[kScanThreads / 32 + 1];
	size_t i = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
	uint4 v = loadTile4(in, n, i, aligned);
	unsigned int s = v.x + v.y + v.z + v.w;
	unsigned int total;
	blockExclusiveScan<kScanThreads>(s, smem, &total);
	if (threadIdx.x == 0)
		sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) kScanApply(const unsigned int* in, unsigned int* out, size_t n, const unsigned int* __restrict__ tileoffs,
    unsigned int* total, bool aligned, const unsigned int* n_dev = nullptr)
{
	__shared__ unsigned int smem[kScanThreads / 32 + 1];
	if (n_dev && *n_dev < n)
		n = *n_dev;
	size_t i = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
	uint4 v = loadTile4(in, n, i, aligned);
	unsigned int s = v.x + v.y + v.z + v.w;
	unsigned int btotal;
	unsigned int pre = blockExclusiveScan<kScanThreads>(s, smem, &btotal);
	unsigned int base = tileoffs ? tileoffs[blockIdx.x] : 0u;
	pre += base;
	uint4 o;
	o.x = pre;
	o.y = o.x + v.x;
	o.z = o.y + v.y;
	o.w = o.z + v.z;
	if (aligned && i + 3 < n)
		*reinterpret_cast<uint4*>(out + i) = o;
	else
	{
		if (i + 0 < n)
			out[i + 0] = o.x;
		if (i + 1 < n)
			out[i + 1] = o.y;
		if (i + 2 < n)
			out[i + 2] = o.z;
		if (i + 3 < n)
			out[i + 3] = o.w;
	}
	if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
		*total = base + btotal;
}

// The whole scan in one cooperative launch: block b reduces its run of consecutive tiles into
// sums[b]; after the grid barrier each block adds up the sums before it and scans its tiles
// again, writing the prefixes. in and out may alias: a block writes only elements it has read.
__global__ void __launch_bounds__(kScanThreads) kScanCoop(const unsigned int* in, unsigned int* out, size_t n, unsigned int* total,
    unsigned int* sums, unsigned int* bar, unsigned int* err, bool aligned, const unsigned int* n_dev)
{
	__shared__ unsigned int smem[kScanThreads / 32 + 1];
	if (n_dev && *n_dev < n)
		n = *n_dev; // the live count; the grid covers n
	const size_t tiles = (n + kScanTile - 1) / kScanTile;
	const size_t per = (tiles + gridDim.x - 1) / gridDim.x;
	const size_t t0 = min(tiles, (size_t)blockIdx.x * per), t1 = min(tiles, t0 + per);
	unsigned int s = 0;
	for (size_t t = t0; t < t1; ++t)
	{
		const uint4 v = loadTile4(in, n, t * kScanTile + (size_t)threadIdx.x * kScanItems, aligned);
		s += v.x + v.y + v.z + v.w;
	}
	unsigned int part;
	blockExclusiveScan<kScanThreads>(s, smem, &part);
	if (threadIdx.x == 0)
		sums[blockIdx.x] = part;
	gridBarrierOnce(bar, err);
	if (__ldcg(err))
		return; // a barrier wait ran out: no block writes prefixes from incomplete sums
	unsigned int before = 0;
	for (unsigned int j = threadIdx.x; j < blockIdx.x; j += kScanThreads)
		before += __ldcg(sums + j);
	unsigned int base;
	blockExclusiveScan<kScanThreads>(before, smem, &base);
	for (size_t t = t0; t < t1; ++t)
	{
		const size_t i = t * kScanTile + (size_t)threadIdx.x * kScanItems;
		const uint4 v = loadTile4(in, n, i, aligned);
		__syncthreads(); // every thread has read the previous scan's shared words
		unsigned int tile_total;
		const unsigned int pre = base + blockExclusiveScan<kScanThreads>(v.x + v.y + v.z + v.w, smem, &tile_total);
		uint4 o;
		o.x = pre;
		o.y = o.x + v.x;
		o.z = o.y + v.y;
		o.w = o.z + v.z;
		if (aligned && i + 3 < n)
			*reinterpret_cast<uint4*>(out + i) = o;
		else
		{
			if (i + 0 < n)
				out[i + 0] = o.x;
			if (i + 1 < n)
				out[i + 1] = o.y;
			if (i + 2 < n)
				out[i + 2] = o.z;
			if (i + 3 < n)
				out[i + 3] = o.w;
		}
		base += tile_total;
	}
	if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
		*total = base;
}

size_t roundWords(size_t w)
{
	return (w + 63) & ~size_t(63);
}

void scanLevel(const unsigned int* in, unsigned int* out, size_t n, unsigned int* total, unsigned int* scratch, cudaStream_t stream, ScanSync sync)
{
	size_t tiles = (n + kScanTile - 1) / kScanTile;
	bool aligned = ((uintptr_t)in % 16 == 0) && ((uintptr_t)out % 16 == 0);
	if (tiles <= 1)
	{
		MO_LAUNCH(kScanApply, 1, kScanThreads, 0, stream, in, out, n, nullptr, total, aligned, sync.n_dev);
		return;
	}
	unsigned int cap = sync.bar ? coopScanCapacity() : 0u;
	if (cap && sync.max_blocks)
		cap = std::min(cap, sync.max_blocks);
	if (sync.n_dev && !cap)
		throw std::invalid_argument("scanExclusive: a device-side count needs the single-launch mode");
	if (cap)
	{
		// consecutive tiles per block, then as few blocks as that needs
		const size_t per = (tiles + cap - 1) / cap;
		const unsigned int blocks = unsigned((tiles + per - 1) / per);
		unsigned int* sums = scratch;
		cudaEvent_t e0 = probeBegin("kScanCoop", stream);
		void* params[] = {(void*)&in, (void*)&out, (void*)&n, (void*)&total, (void*)&sums, (void*)&sync.bar, (void*)&sync.err, (void*)&aligned,
		                  (void*)&sync.n_dev};
		MO_CUDA_CHECK(cudaLaunchCooperativeKernel((const void*)kScanCoop, dim3(blocks), dim3(kScanThreads), params, 0, stream));
		probeEnd(e0, stream);
		return;
	}
	unsigned int* sums = scratch;
	MO_LAUNCH(kScanReduce, (unsigned)tiles, kScanThreads, 0, stream, in, n, sums, aligned);
	scanLevel(sums, sums, tiles, nullptr, scratch + roundWords(tiles), stream, ScanSync());
	MO_LAUNCH(kScanApply, (unsigned)tiles, kScanThreads, 0, stream, in, out, n, sums, total, aligned);
}

// n_dev (optional): the live element count on the device, at most n; the grid covers n
__device__ __forceinline__ size_t liveCount(size_t n, const unsigned int* n_dev)
{
	if (!n_dev)
		return n;
	size_t d = *n_dev;
	return d < n ? d : n;
}

__global__ void __launch_bounds__(kSortThreads) kRadixHist(const unsigned int* __restrict__ keys, size_t n, const unsigned int* n_dev, int shift,
    unsigned int* __restrict__ hist, unsigned int tiles)
{
	__shared__ unsigned int sh[kSortBins];
	n = liveCount(n, n_dev);
	sh[threadIdx.x] = 0;
	__syncthreads();
	size_t base = (size_t)blockIdx.x * kSortTile + threadIdx.x;
#pragma unroll 4
	for (int j = 0; j < kSortItems; ++j)
	{
		size_t i = base + (size_t)j * kSortThreads;
		if (i < n)
			atomicAdd(&sh[(__ldg(keys + i) >> shift) & 0xFFu], 1u);
	}
	__syncthreads();
	hist[(size_t)threadIdx.x * tiles + blockIdx.x] = sh[threadIdx.x];
}

// Stable scatter. Warp w ranks the tile's kSortWarpSpan consecutive elements from w*kSortWarpSpan
// on, 32 at a time (lane order within each step, steps in order), against per-warp digit
// counters in shared memory; the warp counters of each digit are then turned into offsets in
// warp order. So equal digits keep their
// input order, and the tile is put in digit order in shared memory with one block barrier per
// phase, then written out front to back: each digit's elements of the tile leave as one
// contiguous run (coalesced stores) at the position the digit-major scanned histogram gives.
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortWarpSpan = kSortTile / kSortWarps; // consecutive elements per warp

__global__ void __launch_bounds__(kSortThreads, 5) kRadixScatter(const unsigned int* __restrict__ kin, const unsigned int* __restrict__ vin,
    unsigned int* __restrict__ kout, unsigned int* __restrict__ vout, size_t n, const unsigned int* n_dev, int shift, const unsigned int* __restrict__ hist,
    unsigned int tiles)
{
	// vin == nullptr stands for the identity values 0..n-1
	n = liveCount(n, n_dev);
	__shared__ unsigned int lbase[kSortBins];              // tile-local start per digit
	__shared__ unsigned int gbase[kSortBins];              // global position of the tile's first element per digit
	__shared__ unsigned int wcnt[kSortWarps][kSortBins];   // per warp and digit: count, then offset within the digit
	__shared__ unsigned int sk[kSortTile], sv[kSortTile];
	__shared__ unsigned int scan_smem[kSortWarps + 1];

	const unsigned int t = threadIdx.x, w = t >> 5, lane = t & 31;
	const size_t tile0 = (size_t)blockIdx.x * kSortTile;
	if (tile0 >= n)
		return;
	const unsigned int tile_n = (unsigned int)min((size_t)kSortTile, n - tile0);
	{
		// the tile's count of digit t: the scanned histogram's next entry (digit-major, so the
		// entry after (t, last tile) is (t + 1, first tile); after the last one comes n)
		const size_t at = (size_t)t * tiles + blockIdx.x;
		const unsigned int g = hist[at];
		const unsigned int next = at + 1 < (size_t)kSortBins * tiles ? hist[at + 1] : (unsigned int)n;
		gbase[t] = g;
		unsigned int total;
		lbase[t] = blockExclusiveScan<kSortThreads>(next - g, scan_smem, &total);
	}
#pragma unroll
	for (int q = 0; q < kSortWarps; ++q)
		wcnt[q][t] = 0;
	__syncthreads();

	// rank within the warp: the digit's count before this element among the warp's elements
	constexpr int kSteps = kSortWarpSpan / 32;
	unsigned int kr[kSteps], rr[kSteps];
	const size_t w0 = tile0 + (size_t)w * kSortWarpSpan + lane;
#pragma unroll
	for (int j = 0; j < kSteps; ++j)
	{
		const size_t i = w0 + (size_t)j * 32;
		kr[j] = i < n ? __ldg(kin + i) : 0u;
	}
#pragma unroll
	for (int j = 0; j < kSteps; ++j)
	{
		const bool valid = w0 + (size_t)j * 32 < n;
		const unsigned int d = valid ? ((kr[j] >> shift) & 0xFFu) : (0x100u + lane);
		const unsigned int peers = __match_any_sync(0xffffffffu, d);
		const unsigned int leader = __ffs(peers) - 1;
		unsigned int before = 0;
		if (valid && lane == leader)
		{
			before = wcnt[w][d];
			wcnt[w][d] = before + __popc(peers);
		}
		before = __shfl_sync(0xffffffffu, before, leader);
		rr[j] = before + __popc(peers & ((1u << lane) - 1u));
		__syncwarp();
	}
	__syncthreads();
	{
		// warp counts of digit t to offsets within the digit, in warp order
		unsigned int run = 0;
#pragma unroll
		for (int q = 0; q < kSortWarps; ++q)
		{
			const unsigned int c = wcnt[q][t];
			wcnt[q][t] = run;
			run += c;
		}
	}
	__syncthreads();
	// the values are loaded only now (fewer registers live through the ranking)
#pragma unroll
	for (int j = 0; j < kSteps; ++j)
	{
		const size_t i = w0 + (size_t)j * 32;
		if (i < n)
		{
			const unsigned int d = (kr[j] >> shift) & 0xFFu;
			const unsigned int lp = lbase[d] + wcnt[w][d] + rr[j];
			sk[lp] = kr[j];
			sv[lp] = vin ? __ldg(vin + i) : (unsigned int)i;
		}
	}
	__syncthreads();
	for (unsigned int x = t; x < tile_n; x += kSortThreads)
	{
		unsigned int k = sk[x];
		unsigned int d = (k >> shift) & 0xFFu;
		unsigned int pos = gbase[d] + (x - lbase[d]);
		kout[pos] = k;
		vout[pos] = sv[x];
	}
}

} // namespace

// The bounded waits of both grid barriers, made to run out: block 0 never arrives, so every
// other block waits `limit` times, records the error and leaves. Nothing faults or hangs.
__global__ void kBarrierWaitProbe(unsigned int* words, unsigned int limit, int once)
{
	if (blockIdx.x == 0)
		return;
	if (once)
		gridBarrierOnce(words, words + 2, limit);
	else
		gridBarrier(words, words + 2, limit);
}

unsigned int probeBarrierWait(int once, unsigned int blocks, unsigned int limit, cudaStream_t stream)
{
	unsigned int* words = nullptr;
	MO_CUDA_CHECK(cudaMalloc(&words, 4 * sizeof(unsigned int)));
	unsigned int err = 0;
	try
	{
		MO_CUDA_CHECK(cudaMemsetAsync(words, 0, 4 * sizeof(unsigned int), stream));
		void* params[] = {(void*)&words, (void*)&limit, (void*)&once};
		cudaEvent_t e0 = probeBegin("kBarrierWaitProbe", stream);
		MO_CUDA_CHECK(cudaLaunchCooperativeKernel((const void*)kBarrierWaitProbe, dim3(blocks), dim3(kScanThreads), params, 0, stream));
		probeEnd(e0, stream);
		MO_CUDA_CHECK(cudaMemcpyAsync(&err, words + 2, sizeof(err), cudaMemcpyDeviceToHost, stream));
		MO_CUDA_CHECK(cudaStreamSynchronize(stream));
	}
	catch (...)
	{
		cudaFree(words);
		throw;
	}
	MO_CUDA_CHECK(cudaFree(words));
	return err;
}

constexpr int kMaxDevices = 64;
constexpr unsigned int kCoopScanBlocksPerSM = 4; // at most this many per SM (occupancy permitting)

unsigned int coopScanCapacity()
{
	static std::atomic<unsigned int> cache[kMaxDevices];
	int dev = 0;
	MO_CUDA_CHECK(cudaGetDevice(&dev));
	if (dev < 0 || dev >= kMaxDevices)
		return 0;
	unsigned int c = cache[dev].load(std::memory_order_relaxed);
	if (c)
		return c;
	int sms = 0, occ = 0;
	MO_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	MO_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kScanCoop, kScanThreads, 0));
	c = unsigned(std::max(1, sms)) * std::min(unsigned(std::max(1, occ)), kCoopScanBlocksPerSM);
	cache[dev].store(c, std::memory_order_relaxed);
	return c;
}

size_t scanScratchWords(size_t n)
{
	size_t words = 64;
	size_t tiles = (n + kScanTile - 1) / kScanTile;
	while (tiles > 1)
	{
		words += roundWords(tiles);
		tiles = (tiles + kScanTile - 1) / kScanTile;
	}
	return words;
}

void scanExclusive(const unsigned int* in, unsigned int* out, size_t n, unsigned int* total, unsigned int* scratch, cudaStream_t stream,
    ScanSync sync)
{
	if (n == 0)
	{
		if (total)
			MO_CUDA_CHECK(cudaMemsetAsync(total, 0, sizeof(unsigned int), stream));
		return;
	}
	scanLevel(in, out, n, total, scratch, stream, sync);
	MO_CUDA_CHECK(cudaGetLastError());
}

size_t radixScratchWords(size_t n)
{
	size_t tiles = (n + kSortTile - 1) / kSortTile;
	size_t h = roundWords(tiles * kSortBins);
	return h + scanScratchWords(tiles * kSortBins);
}

// A sort of at most kSmallSortMax pairs in one block: each pair becomes the 64-bit word
// (key digits << 32 | input position), and a bitonic network sorts the words in shared memory.
// Distinct positions make the order total, so equal keys keep their input order: the result is
// the stable order the digit passes give. The key digits are the low `mask` bits the digit
// passes would look at; keys and values are read back from the input by position.
constexpr unsigned int kSmallSortMax = 4096;
constexpr unsigned int kSmallSortThreads = 1024;

__global__ void __launch_bounds__(kSmallSortThreads) kSmallSortPairs(const unsigned int* __restrict__ kin, const unsigned int* __restrict__ vin,
    unsigned int* __restrict__ kout, unsigned int* __restrict__ vout, unsigned int n, unsigned int mask)
{
	__shared__ unsigned long long s[kSmallSortMax];
	unsigned int m = 1;
	while (m < n)
		m <<= 1;
	for (unsigned int i = threadIdx.x; i < m; i += blockDim.x)
		s[i] = i < n ? ((unsigned long long)(__ldg(kin + i) & mask) << 32) | i : ~0ull;
	__syncthreads();
	for (unsigned int k = 2; k <= m; k <<= 1)
		for (unsigned int j = k >> 1; j > 0; j >>= 1)
		{
			for (unsigned int t = threadIdx.x; t < m / 2; t += blockDim.x)
			{
				const unsigned int lo = 2 * t - (t & (j - 1)), hi = lo + j; // the pair t of this step, lo's bit j clear
				const unsigned long long a = s[lo], b = s[hi];
				if ((a > b) == ((lo & k) == 0))
					s[lo] = b, s[hi] = a;
			}
			__syncthreads();
		}
	for (unsigned int i = threadIdx.x; i < n; i += blockDim.x)
	{
		const unsigned int src = (unsigned int)s[i];
		kout[i] = __ldg(kin + src);
		vout[i] = vin ? __ldg(vin + src) : src;
	}
}

void radixSortPairs(const unsigned int* keys_in, const unsigned int* vals_in, unsigned int* keys_out, unsigned int* vals_out,
    unsigned int* keys_tmp, unsigned int* vals_tmp, size_t n, int bits, unsigned int* scratch, cudaStream_t stream, const unsigned int* n_dev,
    ScanSync sync)
{
	if (n == 0)
		return;
	int passes = (bits + 7) / 8;
	if (passes == 0)
	{
		if (n_dev)
			throw std::invalid_argument("radixSortPairs: a device count needs at least one digit pass");
		MO_CUDA_CHECK(cudaMemcpyAsync(keys_out, keys_in, n * 4, cudaMemcpyDeviceToDevice, stream));
		MO_CUDA_CHECK(cudaMemcpyAsync(vals_out, vals_in, n * 4, cudaMemcpyDeviceToDevice, stream));
		return;
	}
	if (!n_dev && n <= kSmallSortMax)
	{
		const unsigned int mask = passes >= 4 ? ~0u : (1u << (8 * passes)) - 1u;
		MO_LAUNCH(kSmallSortPairs, 1, kSmallSortThreads, 0, stream, keys_in, vals_in, keys_out, vals_out, (unsigned int)n, mask);
		return;
	}
	unsigned int tiles = unsigned((n + kSortTile - 1) / kSortTile);
	unsigned int* hist = scratch;
	unsigned int* sscratch = scratch + roundWords(size_t(tiles) * kSortBins);

	const unsigned int* ks = keys_in;
	const unsigned int* vs = vals_in;
	for (int p = 0; p < passes; ++p)
	{
		// the last pass must land in *_out: pick the destination by parity from the end
		bool to_out = ((passes - 1 - p) % 2) == 0;
		unsigned int* kd = to_out ? keys_out : keys_tmp;
		unsigned int* vd = to_out ? vals_out : vals_tmp;
		int shift = p * 8;
		MO_LAUNCH(kRadixHist, tiles, kSortThreads, 0, stream, ks, n, n_dev, shift, hist, tiles);
		scanExclusive(hist, hist, size_t(tiles) * kSortBins, nullptr, sscratch, stream, sync);
		MO_LAUNCH(kRadixScatter, tiles, kSortThreads, 0, stream, ks, vs, kd, vd, n, n_dev, shift, hist, tiles);
		ks = kd;
		vs = vd;
	}
	MO_CUDA_CHECK(cudaGetLastError());
}

// ---------------------------------------------------------------- launch probe

LaunchProbe::~LaunchProbe()
{
	for (auto& pr : pending)
	{
		cudaEventDestroy(pr.first);
		cudaEventDestroy(pr.second);
	}
	for (cudaEvent_t e : pool)
		cudaEventDestroy(e);
}

cudaEvent_t LaunchProbe::take()
{
	if (!pool.empty())
	{
		cudaEvent_t e = pool.back();
		pool.pop_back();
		return e;
	}
	cudaEvent_t e = nullptr;
	cudaEventCreate(&e);
	return e;
}

void LaunchProbe::collect()
{
	for (auto& pr : pending)
	{
		float ms = 0;
		if (cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess)
		{
			timed_ms += ms;
			timed_launches++;
		}
		pool.push_back(pr.first);
		pool.push_back(pr.second);
	}
	pending.clear();
}

LaunchProbe& probe()
{
	static thread_local LaunchProbe p;
	return p;
}

} // namespace mogpu
