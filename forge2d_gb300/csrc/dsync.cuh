// Device-wide synchronisation primitives shared by the persistent kernels.
//
// grid_barrier: for cooperative launches only (co-residency of every block
// is guaranteed by cudaLaunchCooperativeKernel). One monotonically
// increasing arrival counter, zeroed on the stream before the launch:
// barrier number e is passed when the counter reaches e x gridDim.x. Thread 0
// of each block publishes the block's writes with a release add and waits
// with acquire loads; __syncthreads orders the rest of the block on either
// side. Shared data written before a barrier is read after it with L2 (.cg)
// or acquire loads, so no stale L1 line survives. Every wait is bounded: a
// block that gives up sets the timeout bit in *err and every other block
// leaves at its next poll of that word.
#pragma once

#include <cuda_runtime.h>

#define F2D_SPIN_LIMIT ( 1ll << 24 )
#define F2D_ERR_BARRIER_TIMEOUT 0x4

__device__ __forceinline__ void red_release_add( unsigned* p, unsigned v )
{
	asm volatile( "red.release.gpu.global.add.u32 [%0], %1;" ::"l"( p ), "r"( v ) : "memory" );
}

__device__ __forceinline__ unsigned ld_acquire_u32( const unsigned* p )
{
	unsigned v;
	asm volatile( "ld.acquire.gpu.global.u32 %0, [%1];" : "=r"( v ) : "l"( p ) : "memory" );
	return v;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64( const unsigned long long* p )
{
	unsigned long long v;
	asm volatile( "ld.acquire.gpu.global.u64 %0, [%1];" : "=l"( v ) : "l"( p ) : "memory" );
	return v;
}

__device__ __forceinline__ void st_release_u64( unsigned long long* p, unsigned long long v )
{
	asm volatile( "st.release.gpu.global.u64 [%0], %1;" ::"l"( p ), "l"( v ) : "memory" );
}

__device__ __forceinline__ int ld_relaxed_s32( const int* p )
{
	int v;
	asm volatile( "ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"( v ) : "l"( p ) : "memory" );
	return v;
}

// counter: zeroed before the launch; epoch: barriers this block has passed
// in this launch (identical on every block). Returns false on timeout.
__device__ __forceinline__ bool grid_barrier( unsigned* counter, int* err, unsigned& epoch )
{
	__shared__ int s_timedOut;
	__syncthreads();
	epoch += 1;
	if ( threadIdx.x == 0 )
	{
		unsigned target = epoch * gridDim.x;
		red_release_add( counter, 1u );
		long long spins = 0;
		int timedOut = 0;
		while ( (int)( ld_acquire_u32( counter ) - target ) < 0 )
		{
			++spins;
			if ( spins > F2D_SPIN_LIMIT ||
				 ( ( spins & 1023 ) == 0 && ( ld_relaxed_s32( err ) & F2D_ERR_BARRIER_TIMEOUT ) ) )
			{
				atomicOr( err, F2D_ERR_BARRIER_TIMEOUT );
				timedOut = 1;
				break;
			}
		}
		s_timedOut = timedOut;
	}
	__syncthreads();
	return s_timedOut == 0;
}
