// Device-count-driven exclusive scan and stable LSD radix sort.
//
// Element counts live in device memory, so every launch has a fixed grid
// sized from a capacity and the whole step can be enqueued (and captured in
// a CUDA graph) without host round trips. Blocks beyond the live count exit
// after reading it.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define SCAN_THREADS 1024
#define SCAN_ITEMS 4
#define SCAN_TILE ( SCAN_THREADS * SCAN_ITEMS )

#define SORT_THREADS 256
#define SORT_CHUNKS 16
#define SORT_TILE ( SORT_THREADS * SORT_CHUNKS )
#define SORT_WARPS ( SORT_THREADS / 32 )

__device__ __forceinline__ int block_exclusive_scan_1024( int v, int* smem, int* total )
{
	// warp-level inclusive scan then a scan of warp totals (32 warps)
	int lane = threadIdx.x & 31;
	int warp = threadIdx.x >> 5;
	int x = v;
#pragma unroll
	for ( int o = 1; o < 32; o <<= 1 )
	{
		int y = __shfl_up_sync( 0xffffffffu, x, o );
		if ( lane >= o )
			x += y;
	}
	if ( lane == 31 )
		smem[warp] = x;
	__syncthreads();
	if ( warp == 0 )
	{
		int nw = ( blockDim.x + 31 ) >> 5;
		int w = lane < nw ? smem[lane] : 0;
#pragma unroll
		for ( int o = 1; o < 32; o <<= 1 )
		{
			int y = __shfl_up_sync( 0xffffffffu, w, o );
			if ( lane >= o )
				w += y;
		}
		smem[lane] = w; // inclusive warp totals
	}
	__syncthreads();
	int warpBase = warp > 0 ? smem[warp - 1] : 0;
	int excl = warpBase + x - v;
	if ( total )
		*total = smem[( ( blockDim.x + 31 ) >> 5 ) - 1];
	__syncthreads();
	return excl;
}

// per-tile exclusive scan; writes tile sums
static __global__ void k_scan_tiles( const int* __restrict__ in, int* __restrict__ out, int* __restrict__ tileSums,
							  const int* __restrict__ nPtr, int nConst )
{
	__shared__ int smem[32];
	int n = nPtr ? *nPtr : nConst;
	int base = blockIdx.x * SCAN_TILE;
	if ( base >= n )
	{
		if ( threadIdx.x == 0 )
			tileSums[blockIdx.x] = 0;
		return;
	}
	int v[SCAN_ITEMS];
	int sum = 0;
#pragma unroll
	for ( int k = 0; k < SCAN_ITEMS; ++k )
	{
		int i = base + threadIdx.x * SCAN_ITEMS + k;
		v[k] = i < n ? in[i] : 0;
		sum += v[k];
	}
	int total;
	int excl = block_exclusive_scan_1024( sum, smem, &total );
#pragma unroll
	for ( int k = 0; k < SCAN_ITEMS; ++k )
	{
		int i = base + threadIdx.x * SCAN_ITEMS + k;
		if ( i < n )
			out[i] = excl;
		excl += v[k];
	}
	if ( threadIdx.x == 0 )
		tileSums[blockIdx.x] = total;
}

// single block scans up to SCAN_TILE tile sums in place; optional grand total
static __global__ void k_scan_sums( int* __restrict__ sums, int count, int* __restrict__ totalOut )
{
	__shared__ int smem[32];
	int v[SCAN_ITEMS];
	int sum = 0;
#pragma unroll
	for ( int k = 0; k < SCAN_ITEMS; ++k )
	{
		int i = threadIdx.x * SCAN_ITEMS + k;
		v[k] = i < count ? sums[i] : 0;
		sum += v[k];
	}
	int total;
	int excl = block_exclusive_scan_1024( sum, smem, &total );
#pragma unroll
	for ( int k = 0; k < SCAN_ITEMS; ++k )
	{
		int i = threadIdx.x * SCAN_ITEMS + k;
		if ( i < count )
			sums[i] = excl;
		excl += v[k];
	}
	if ( threadIdx.x == 0 && totalOut )
		*totalOut = total;
}

static __global__ void k_scan_add( int* __restrict__ out, const int* __restrict__ tileSums, const int* __restrict__ nPtr,
							int nConst )
{
	int n = nPtr ? *nPtr : nConst;
	int base = blockIdx.x * SCAN_TILE;
	if ( base >= n )
		return;
	int add = tileSums[blockIdx.x];
#pragma unroll
	for ( int k = 0; k < SCAN_ITEMS; ++k )
	{
		int i = base + threadIdx.x * SCAN_ITEMS + k;
		if ( i < n )
			out[i] += add;
	}
}

// Exclusive scan of n ints (n read from nPtr when non-null, else nConst);
// capacity bounds the grid. tmp needs cap/SCAN_TILE+1 ints. totalOut (device)
// receives the sum when non-null.
static inline void scan_exclusive( const int* in, int* out, int* tmp, const int* nPtr, int nConst, int cap,
								   int* totalOut, cudaStream_t st )
{
	int tiles = ( cap + SCAN_TILE - 1 ) / SCAN_TILE;
	if ( tiles < 1 )
		tiles = 1;
	k_scan_tiles<<<tiles, SCAN_THREADS, 0, st>>>( in, out, tmp, nPtr, nConst );
	k_scan_sums<<<1, SCAN_THREADS, 0, st>>>( tmp, tiles, totalOut );
	k_scan_add<<<tiles, SCAN_THREADS, 0, st>>>( out, tmp, nPtr, nConst );
}

template <typename K>
__global__ void k_radix_hist( const K* __restrict__ keys, const int* __restrict__ nPtr, int shift,
							  unsigned* __restrict__ hist, int numBlocks )
{
	__shared__ unsigned h[256];
	int n = *nPtr;
	h[threadIdx.x] = 0;
	__syncthreads();
	int base = blockIdx.x * SORT_TILE;
	for ( int c = 0; c < SORT_CHUNKS; ++c )
	{
		int i = base + c * SORT_THREADS + threadIdx.x;
		if ( i < n )
		{
			unsigned d = (unsigned)( ( keys[i] >> shift ) & 0xff );
			atomicAdd( h + d, 1u );
		}
	}
	__syncthreads();
	hist[threadIdx.x * numBlocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: elements keep their input order within equal digits
// (tile order, then chunk order, then warp, then lane).
template <typename K>
__global__ void k_radix_scatter( const K* __restrict__ keys, const int* __restrict__ vals, K* __restrict__ keysOut,
								 int* __restrict__ valsOut, const int* __restrict__ nPtr, int shift,
								 const unsigned* __restrict__ offsets, int numBlocks )
{
	__shared__ unsigned base[256];
	__shared__ unsigned warpHist[SORT_WARPS][256];
	int n = *nPtr;
	int tileBase = blockIdx.x * SORT_TILE;
	if ( tileBase >= n )
		return;
	base[threadIdx.x] = offsets[threadIdx.x * numBlocks + blockIdx.x];
	int lane = threadIdx.x & 31;
	int warp = threadIdx.x >> 5;
	for ( int c = 0; c < SORT_CHUNKS; ++c )
	{
		for ( int w = 0; w < SORT_WARPS; ++w )
			warpHist[w][threadIdx.x] = 0;
		__syncthreads();
		int i = tileBase + c * SORT_THREADS + threadIdx.x;
		bool valid = i < n;
		K key = valid ? keys[i] : (K)0;
		int val = valid ? vals[i] : 0;
		unsigned d = valid ? (unsigned)( ( key >> shift ) & 0xff ) : ( 256u + (unsigned)lane );
		unsigned peers = __match_any_sync( 0xffffffffu, d );
		unsigned rankInWarp = __popc( peers & ( ( 1u << lane ) - 1u ) );
		if ( valid && rankInWarp == 0 )
			warpHist[warp][d] = __popc( peers );
		__syncthreads();
		// thread t owns digit t: exclusive prefix over warps, then advance base
		{
			unsigned run = 0;
			for ( int w = 0; w < SORT_WARPS; ++w )
			{
				unsigned t = warpHist[w][threadIdx.x];
				warpHist[w][threadIdx.x] = run;
				run += t;
			}
			// stash chunk total in the register; base updated after use
			__syncthreads();
			if ( valid )
			{
				unsigned dst = base[d] + warpHist[warp][d] + rankInWarp;
				keysOut[dst] = key;
				valsOut[dst] = val;
			}
			__syncthreads();
			base[threadIdx.x] += run;
		}
		__syncthreads();
	}
}

// Sorts (keys, vals) ascending by the low `bits` bits of the keys, in place
// (alt buffers are scratch). n from device memory; cap bounds the grid.
// histTmp needs 256*blocks + SCAN sums space.
template <typename K>
static inline void radix_sort( K* keys, int* vals, K* keysAlt, int* valsAlt, const int* nPtr, int cap, int bits,
							   unsigned* hist, int* scanTmp, cudaStream_t st )
{
	int blocks = ( cap + SORT_TILE - 1 ) / SORT_TILE;
	if ( blocks < 1 )
		blocks = 1;
	int passes = ( bits + 7 ) / 8;
	if ( passes & 1 )
		passes += 1; // even pass count leaves the result in the input buffers
	K* kin = keys;
	int* vin = vals;
	K* kout = keysAlt;
	int* vout = valsAlt;
	for ( int p = 0; p < passes; ++p )
	{
		int shift = 8 * p;
		if ( shift >= (int)( 8 * sizeof( K ) ) )
			shift = 8 * (int)sizeof( K ) - 8; // extra pass re-sorts the top digit (stable, no-op)
		k_radix_hist<K><<<blocks, SORT_THREADS, 0, st>>>( kin, nPtr, shift, hist, blocks );
		scan_exclusive( (const int*)hist, (int*)hist, scanTmp, nullptr, 256 * blocks, 256 * blocks, nullptr, st );
		k_radix_scatter<K><<<blocks, SORT_THREADS, 0, st>>>( kin, vin, kout, vout, nPtr, shift, hist, blocks );
		K* tk = kin;
		kin = kout;
		kout = tk;
		int* tv = vin;
		vin = vout;
		vout = tv;
	}
}
