// One-launch device sort and scan for the world step.
//
// Element counts live in device memory (the step is enqueued without host
// round trips), so the launch shapes are fixed and each kernel reads n
// itself.
//
// * sort_coop: stable LSD radix sort of (key, value) rows by the low `bits`
//   bits of the key, as ONE cooperative launch: per 8-bit digit, a block
//   histogram, a grid barrier, per-block digit offsets, a stable scatter
//   (warp match_any ranks) and another grid barrier. Rows of n <= SMALL are
//   sorted by block 0 alone in shared memory (bitonic on (key, value), which
//   is the same order the stable sort gives when the input values ascend).
// * scan_lookback: exclusive scan of n ints in one launch (decoupled
//   look-back across tiles claimed in launch order).
#pragma once

#include "dscan.cuh"
#include "dsync.cuh"

#include <climits>

#define CSORT_THREADS 1024
#define CSORT_SMALL 2048
#define CSORT_MAX_BLOCKS 256
#define CSORT_WARPS ( CSORT_THREADS / 32 )

#define LB_THREADS 1024
#define LB_ITEMS 8
#define LB_TILE ( LB_THREADS * LB_ITEMS )
#define LB_FLAG_AGG 1ull
#define LB_FLAG_PREFIX 2ull

template <typename K> __device__ __forceinline__ bool kv_less( K ka, int va, K kb, int vb )
{
	return ka < kb || ( ka == kb && va < vb );
}

// shared memory of k_sort_coop: the bitonic buffers or the radix tables
union CSortSmem
{
	struct
	{
		unsigned long long key[CSORT_SMALL];
		int val[CSORT_SMALL];
	} small;
	struct
	{
		unsigned base[256];				   // running scatter base per digit
		unsigned warpHist[CSORT_WARPS][256]; // per-warp digit counts, then prefixes
		unsigned partTotal[4][256];		   // digit totals per quarter of the blocks
		unsigned partBefore[4][256];	   // same, only blocks before this one
		int scan[32];
	} radix;
};

template <typename K>
__global__ void __launch_bounds__( CSORT_THREADS )
	k_sort_coop( K* keys, int* vals, K* keysAlt, int* valsAlt, const int* nPtr, int bits, unsigned* hist,
				 unsigned* counter, int* err, const int* enable )
{
	__shared__ CSortSmem sm;
	const int tid = threadIdx.x;
	if ( enable && *enable == 0 )
		return;
	const int n = *nPtr;
	if ( n <= 1 )
		return;
	if ( n <= CSORT_SMALL )
	{
		if ( blockIdx.x != 0 )
			return;
		int P = 2;
		while ( P < n )
			P <<= 1;
		for ( int i = tid; i < P; i += CSORT_THREADS )
		{
			sm.small.key[i] = i < n ? (unsigned long long)keys[i] : ~0ull;
			sm.small.val[i] = i < n ? ( vals ? vals[i] : i ) : INT_MAX;
		}
		__syncthreads();
		for ( int k = 2; k <= P; k <<= 1 )
		{
			for ( int j = k >> 1; j > 0; j >>= 1 )
			{
				for ( int t = tid; t < ( P >> 1 ); t += CSORT_THREADS )
				{
					int i = ( ( t & ~( j - 1 ) ) << 1 ) | ( t & ( j - 1 ) );
					int l = i + j;
					unsigned long long ki = sm.small.key[i], kl = sm.small.key[l];
					int vi = sm.small.val[i], vl = sm.small.val[l];
					bool up = ( i & k ) == 0;
					bool swap = up ? kv_less( kl, vl, ki, vi ) : kv_less( ki, vi, kl, vl );
					if ( swap )
					{
						sm.small.key[i] = kl;
						sm.small.key[l] = ki;
						sm.small.val[i] = vl;
						sm.small.val[l] = vi;
					}
				}
				__syncthreads();
			}
		}
		for ( int i = tid; i < n; i += CSORT_THREADS )
		{
			keys[i] = (K)sm.small.key[i];
			if ( vals )
				vals[i] = sm.small.val[i];
		}
		return;
	}

	unsigned epoch = 0;
	const int G = gridDim.x;
	const int per = ( n + G - 1 ) / G;
	const int lo = min( n, blockIdx.x * per ), hi = min( n, lo + per );
	const int lane = tid & 31, warp = tid >> 5;
	const int passes = ( bits + 7 ) / 8;
	// A digit every row shares needs no pass (a stable pass over it keeps
	// the order): the OR and the AND of all keys, one word pair per block in
	// the histogram buffer's last rows, which the histograms of at most
	// CSORT_MAX_BLOCKS - 4 blocks never reach.
	unsigned long long diff = ~0ull;
	if ( G <= CSORT_MAX_BLOCKS - 4 )
	{
		__shared__ unsigned long long sOr, sAnd;
		unsigned long long o = 0ull, a = ~0ull;
		for ( int i = lo + tid; i < hi; i += CSORT_THREADS )
		{
			unsigned long long k = (unsigned long long)__ldcg( keys + i );
			o |= k;
			a &= k;
		}
#pragma unroll
		for ( int off = 16; off > 0; off >>= 1 )
		{
			o |= __shfl_xor_sync( 0xffffffffu, o, off );
			a &= __shfl_xor_sync( 0xffffffffu, a, off );
		}
		if ( tid == 0 )
		{
			sOr = 0ull;
			sAnd = ~0ull;
		}
		__syncthreads();
		if ( lane == 0 )
		{
			atomicOr( &sOr, o );
			atomicAnd( &sAnd, a );
		}
		__syncthreads();
		unsigned long long* part = (unsigned long long*)( hist + 256 * ( CSORT_MAX_BLOCKS - 4 ) );
		if ( tid == 0 )
		{
			__stcg( part + 2 * blockIdx.x, sOr );
			__stcg( part + 2 * blockIdx.x + 1, sAnd );
		}
		if ( !grid_barrier( counter, err, epoch ) )
			return;
		if ( tid == 0 )
		{
			sOr = 0ull;
			sAnd = ~0ull;
		}
		__syncthreads();
		o = 0ull;
		a = ~0ull;
		for ( int b = tid; b < G; b += CSORT_THREADS )
		{
			o |= __ldcg( part + 2 * b );
			a &= __ldcg( part + 2 * b + 1 );
		}
#pragma unroll
		for ( int off = 16; off > 0; off >>= 1 )
		{
			o |= __shfl_xor_sync( 0xffffffffu, o, off );
			a &= __shfl_xor_sync( 0xffffffffu, a, off );
		}
		if ( lane == 0 )
		{
			atomicOr( &sOr, o );
			atomicAnd( &sAnd, a );
		}
		__syncthreads();
		diff = sOr ^ sAnd;
	}
	K* kin = keys;
	int* vin = vals;
	K* kout = keysAlt;
	int* vout = valsAlt;
	int done = 0;
	for ( int p = 0; p < passes; ++p )
	{
		const int shift = 8 * p;
		if ( ( ( diff >> shift ) & 0xffull ) == 0ull )
			continue;
		done += 1;
		// 1. digit histogram of this block's rows
		if ( tid < 256 )
			sm.radix.base[tid] = 0;
		__syncthreads();
		for ( int i = lo + tid; i < hi; i += CSORT_THREADS )
			atomicAdd( sm.radix.base + (unsigned)( ( __ldcg( kin + i ) >> shift ) & 0xff ), 1u );
		__syncthreads();
		if ( tid < 256 )
			hist[blockIdx.x * 256 + tid] = sm.radix.base[tid];
		if ( !grid_barrier( counter, err, epoch ) )
			return;
		// 2. this block's first output position per digit: rows of smaller
		// digits anywhere plus rows of this digit in earlier blocks
		{
			int d = tid & 255, q = tid >> 8;
			unsigned total = 0, before = 0;
			for ( int b = q; b < G; b += 4 )
			{
				unsigned v = __ldcg( hist + b * 256 + d );
				total += v;
				before += b < (int)blockIdx.x ? v : 0u;
			}
			sm.radix.partTotal[q][d] = total;
			sm.radix.partBefore[q][d] = before;
		}
		__syncthreads();
		unsigned digitTotal = 0, digitBefore = 0;
		if ( tid < 256 )
		{
			for ( int q = 0; q < 4; ++q )
			{
				digitTotal += sm.radix.partTotal[q][tid];
				digitBefore += sm.radix.partBefore[q][tid];
			}
		}
		int dummy;
		int digitStart = block_exclusive_scan_1024( (int)digitTotal, sm.radix.scan, &dummy );
		if ( tid < 256 )
			sm.radix.base[tid] = (unsigned)digitStart + digitBefore;
		__syncthreads();
		// 3. stable scatter, chunk by chunk in row order
		for ( int c0 = lo; c0 < hi; c0 += CSORT_THREADS )
		{
			int i = c0 + tid;
			bool valid = i < hi;
			K key = valid ? __ldcg( kin + i ) : (K)0;
			int val = ( valid && vin ) ? __ldcg( vin + i ) : 0;
			unsigned d = valid ? (unsigned)( ( key >> shift ) & 0xff ) : ( 256u + (unsigned)lane );
			for ( int k = tid; k < CSORT_WARPS * 256; k += CSORT_THREADS )
				( &sm.radix.warpHist[0][0] )[k] = 0;
			__syncthreads();
			unsigned peers = __match_any_sync( 0xffffffffu, d );
			unsigned rank = __popc( peers & ( ( 1u << lane ) - 1u ) );
			if ( valid && rank == 0 )
				sm.radix.warpHist[warp][d] = __popc( peers );
			__syncthreads();
			unsigned run = 0;
			if ( tid < 256 )
			{
				for ( int w = 0; w < CSORT_WARPS; ++w )
				{
					unsigned t = sm.radix.warpHist[w][tid];
					sm.radix.warpHist[w][tid] = run;
					run += t;
				}
			}
			__syncthreads();
			if ( valid )
			{
				unsigned dst = sm.radix.base[d] + sm.radix.warpHist[warp][d] + rank;
				kout[dst] = key;
				if ( vout )
					vout[dst] = val;
			}
			__syncthreads();
			if ( tid < 256 )
				sm.radix.base[tid] += run;
			__syncthreads();
		}
		if ( !grid_barrier( counter, err, epoch ) )
			return;
		K* tk = kin;
		kin = kout;
		kout = tk;
		int* tv = vin;
		vin = vout;
		vout = tv;
	}
	if ( done & 1 )
	{
		// the rows ended in the alternate buffers: copy this block's range back
		for ( int i = lo + tid; i < hi; i += CSORT_THREADS )
		{
			keys[i] = __ldcg( kin + i );
			if ( vals )
				vals[i] = __ldcg( vin + i );
		}
	}
}

// Sorts (keys, vals) by the low `bits` bits of the keys; vals may be null.
// n from device memory. hist needs 256 * CSORT_MAX_BLOCKS unsigned; counter
// is a device word used by the grid barrier (zeroed here). When enable is
// non-null the sort runs only if *enable != 0.
template <typename K>
static inline void sort_coop( K* keys, int* vals, K* keysAlt, int* valsAlt, const int* nPtr, int bits,
							  unsigned* hist, unsigned* counter, int* err, int blocks, cudaStream_t st,
							  const int* enable = nullptr )
{
	if ( blocks > CSORT_MAX_BLOCKS )
		blocks = CSORT_MAX_BLOCKS;
	if ( vals == nullptr )
		valsAlt = nullptr;
	cudaMemsetAsync( counter, 0, sizeof( unsigned ), st );
	void* args[] = { &keys, &vals, &keysAlt, &valsAlt, &nPtr, &bits, &hist, &counter, &err, &enable };
	cudaLaunchCooperativeKernel( (void*)k_sort_coop<K>, dim3( blocks ), dim3( CSORT_THREADS ), args, 0, st );
}

// Co-resident block count for k_sort_coop on the current device.
template <typename K> static inline int sort_coop_blocks()
{
	int perSM = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor( &perSM, k_sort_coop<K>, CSORT_THREADS, 0 );
	int dev = 0, sms = 0;
	cudaGetDevice( &dev );
	cudaDeviceGetAttribute( &sms, cudaDevAttrMultiProcessorCount, dev );
	int b = perSM >= 1 ? sms : 0;
	return b > CSORT_MAX_BLOCKS ? CSORT_MAX_BLOCKS : b;
}

// ---------------------------------------------------------------------------
// exclusive scan with decoupled look-back
// state[0]: tile ticket; state[1 + t]: tile t's flag (bits 32..33) and value
// ---------------------------------------------------------------------------
static __global__ void __launch_bounds__( LB_THREADS )
	k_scan_lookback( const int* __restrict__ in, int* __restrict__ out, const int* __restrict__ nPtr, int nConst,
					 unsigned long long* state, int* __restrict__ totalOut, int* err, const int* enable )
{
	__shared__ int smem[32];
	__shared__ int s_tile, s_prefix;
	if ( enable && *enable == 0 )
		return;
	int n = nPtr ? *nPtr : nConst;
	if ( threadIdx.x == 0 )
		s_tile = (int)atomicAdd( (unsigned*)state, 1u );
	__syncthreads();
	int tile = s_tile;
	int base = tile * LB_TILE;
	if ( base >= n )
	{
		if ( tile == 0 && threadIdx.x == 0 && totalOut )
			*totalOut = 0;
		return;
	}
	int v[LB_ITEMS];
	int sum = 0;
#pragma unroll
	for ( int k = 0; k < LB_ITEMS; ++k )
	{
		int i = base + threadIdx.x * LB_ITEMS + k;
		v[k] = i < n ? in[i] : 0;
		sum += v[k];
	}
	int aggregate;
	int excl = block_exclusive_scan_1024( sum, smem, &aggregate );
	if ( threadIdx.x == 0 )
	{
		int prefix = 0;
		if ( tile == 0 )
			st_release_u64( state + 1, ( LB_FLAG_PREFIX << 32 ) | (unsigned)aggregate );
		else
		{
			st_release_u64( state + 1 + tile, ( LB_FLAG_AGG << 32 ) | (unsigned)aggregate );
			int j = tile - 1;
			long long spins = 0;
			while ( j >= 0 )
			{
				unsigned long long s = ld_acquire_u64( state + 1 + j );
				unsigned long long flag = s >> 32;
				if ( flag == 0ull )
				{
					if ( ++spins > F2D_SPIN_LIMIT )
					{
						atomicOr( err, F2D_ERR_BARRIER_TIMEOUT );
						break;
					}
					continue;
				}
				prefix += (int)(unsigned)( s & 0xffffffffull );
				if ( flag == LB_FLAG_PREFIX )
					break;
				j -= 1;
			}
			st_release_u64( state + 1 + tile, ( LB_FLAG_PREFIX << 32 ) | (unsigned)( prefix + aggregate ) );
		}
		s_prefix = prefix;
		if ( totalOut && base + LB_TILE >= n )
			*totalOut = prefix + aggregate;
	}
	__syncthreads();
	excl += s_prefix;
#pragma unroll
	for ( int k = 0; k < LB_ITEMS; ++k )
	{
		int i = base + threadIdx.x * LB_ITEMS + k;
		if ( i < n )
			out[i] = excl;
		excl += v[k];
	}
}

// Exclusive scan of n ints (n from nPtr when non-null, else nConst); cap
// bounds the grid; state needs cap / LB_TILE + 2 words; totalOut (device)
// receives the sum when non-null. When enable is non-null the scan runs only
// if *enable != 0.
static inline void scan_lookback( const int* in, int* out, const int* nPtr, int nConst, int cap, int* totalOut,
								  unsigned long long* state, int* err, cudaStream_t st,
								  const int* enable = nullptr )
{
	int tiles = ( cap + LB_TILE - 1 ) / LB_TILE;
	if ( tiles < 1 )
		tiles = 1;
	cudaMemsetAsync( state, 0, sizeof( unsigned long long ) * (size_t)( tiles + 1 ), st );
	k_scan_lookback<<<tiles, LB_THREADS, 0, st>>>( in, out, nPtr, nConst, state, totalOut, err, enable );
}
