// Learned warm start: a small MLP [12 -> 64 -> 64 -> 2] that predicts the
// normal and tangent impulses of newly touching manifold points from
// features the contact prepare stage records, trained on impulses the plain
// solver itself produced.
//
// Numerics: BF16 weights and activations into the matrix products, FP32
// accumulation, FP32 master weights and biases (Adam). The products run on
// the tensor cores through warp-level mma.sync m16n8k16 BF16 instructions:
// one warp holds 16 samples, a 64-wide layer is eight 16x8 output tiles.
// The network is 64 wide, so every product is a handful of MMA tiles per
// warp and the kernels are bound by latency, not by tensor throughput.
//
// Layout: W1 [64][16] (12 feature columns, 4 zero columns), W2 [64][64],
// W3 [8][64] (2 output rows, 6 zero rows), row-major by output; b1 [64],
// b2 [64], b3 [8]. Features and targets are normalised with per-column mean
// and 1/std held with the model.
#include "../../include/forge2d_gb300.h"
#include "dworld.cuh"
#include "kernels.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#define MLP_IN 12
#define MLP_IN_PAD 16
#define MLP_H 64
#define MLP_OUT 2
#define MLP_OUT_PAD 8
#define MLP_WARPS 4
#define MLP_THREADS ( 32 * MLP_WARPS )
#define MLP_SAMPLE 14 // 12 features + 2 targets

// parameter vector (FP32 master): W1, W2, W3, b1, b2, b3
#define P_W1 0
#define P_W2 ( P_W1 + MLP_H * MLP_IN_PAD )
#define P_W3 ( P_W2 + MLP_H * MLP_H )
#define P_B1 ( P_W3 + MLP_OUT_PAD * MLP_H )
#define P_B2 ( P_B1 + MLP_H )
#define P_B3 ( P_B2 + MLP_H )
#define P_COUNT ( P_B3 + MLP_OUT_PAD )

struct MlpModel
{
	float* master;			 // P_COUNT
	__nv_bfloat16* wbf;		 // W1, W2, W3 BF16 copies (P_B1 entries)
	float* grad;			 // P_COUNT
	float* m;				 // Adam first moment
	float* v;				 // Adam second moment
	float* norm;			 // mean[14], invStd[14]
	float* loss;			 // device accumulator
	int step;
	bool used;
};

#define MLP_MAX_MODELS 16
static MlpModel s_models[MLP_MAX_MODELS];

// ---------------------------------------------------------------------------
// warp-level BF16 MMA, m16n8k16, FP32 accumulate
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned pack_bf16( float lo, float hi )
{
	__nv_bfloat162 v = __floats2bfloat162_rn( lo, hi );
	return *reinterpret_cast<unsigned*>( &v );
}

__device__ __forceinline__ unsigned pack_pair( const __nv_bfloat16* p )
{
	return *reinterpret_cast<const unsigned*>( p );
}

__device__ __forceinline__ unsigned pack2( __nv_bfloat16 lo, __nv_bfloat16 hi )
{
	__nv_bfloat162 v;
	v.x = lo;
	v.y = hi;
	return *reinterpret_cast<unsigned*>( &v );
}

__device__ __forceinline__ void mma16816( float* d, const unsigned* a, const unsigned* b )
{
	asm volatile( "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
				  "{%8, %9}, {%0, %1, %2, %3};"
				  : "+f"( d[0] ), "+f"( d[1] ), "+f"( d[2] ), "+f"( d[3] )
				  : "r"( a[0] ), "r"( a[1] ), "r"( a[2] ), "r"( a[3] ), "r"( b[0] ), "r"( b[1] ) );
}

// A fragment of a 16x16 tile of a row-major BF16 matrix (ld elements per row)
__device__ __forceinline__ void frag_a( unsigned* a, const __nv_bfloat16* A, int ld, int k0, int lane )
{
	int g = lane >> 2, t = lane & 3;
	a[0] = pack_pair( A + g * ld + k0 + 2 * t );
	a[1] = pack_pair( A + ( g + 8 ) * ld + k0 + 2 * t );
	a[2] = pack_pair( A + g * ld + k0 + 2 * t + 8 );
	a[3] = pack_pair( A + ( g + 8 ) * ld + k0 + 2 * t + 8 );
}

// B fragment (16x8, B[k][n]) when B is stored transposed: Bt[n][k] row-major
__device__ __forceinline__ void frag_b_t( unsigned* b, const __nv_bfloat16* Bt, int ld, int k0, int n0, int lane )
{
	int g = lane >> 2, t = lane & 3;
	b[0] = pack_pair( Bt + ( n0 + g ) * ld + k0 + 2 * t );
	b[1] = pack_pair( Bt + ( n0 + g ) * ld + k0 + 2 * t + 8 );
}

// B fragment when B[k][n] is stored row-major (ld per k row)
__device__ __forceinline__ void frag_b( unsigned* b, const __nv_bfloat16* B, int ld, int k0, int n0, int lane )
{
	int g = lane >> 2, t = lane & 3;
	b[0] = pack2( B[( k0 + 2 * t ) * ld + n0 + g], B[( k0 + 2 * t + 1 ) * ld + n0 + g] );
	b[1] = pack2( B[( k0 + 2 * t + 8 ) * ld + n0 + g], B[( k0 + 2 * t + 9 ) * ld + n0 + g] );
}

// A fragment of the transpose: A[m][k] = S[k][m], S row-major (ld per k row)
__device__ __forceinline__ void frag_a_t( unsigned* a, const __nv_bfloat16* S, int ld, int m0, int lane )
{
	int g = lane >> 2, t = lane & 3;
	a[0] = pack2( S[( 2 * t ) * ld + m0 + g], S[( 2 * t + 1 ) * ld + m0 + g] );
	a[1] = pack2( S[( 2 * t ) * ld + m0 + g + 8], S[( 2 * t + 1 ) * ld + m0 + g + 8] );
	a[2] = pack2( S[( 2 * t + 8 ) * ld + m0 + g], S[( 2 * t + 9 ) * ld + m0 + g] );
	a[3] = pack2( S[( 2 * t + 8 ) * ld + m0 + g + 8], S[( 2 * t + 9 ) * ld + m0 + g + 8] );
}

struct MlpSmem
{
	__nv_bfloat16 w1[MLP_H * MLP_IN_PAD];
	__nv_bfloat16 w2[MLP_H * MLP_H];
	__nv_bfloat16 w3[MLP_OUT_PAD * MLP_H];
	float b1[MLP_H], b2[MLP_H], b3[MLP_OUT_PAD];
	float norm[2 * MLP_SAMPLE];
	// per warp: 16 samples
	__nv_bfloat16 x[MLP_WARPS][16 * MLP_IN_PAD];
	__nv_bfloat16 h1[MLP_WARPS][16 * MLP_H];
	__nv_bfloat16 h2[MLP_WARPS][16 * MLP_H];
	__nv_bfloat16 dz[MLP_WARPS][16 * MLP_H]; // dz2, then dz1
	unsigned char m1[MLP_WARPS][16 * MLP_H]; // relu'(z1): z1 > 0
	unsigned char m2[MLP_WARPS][16 * MLP_H];
	float y[MLP_WARPS][16 * MLP_OUT_PAD];
	float t[MLP_WARPS][16 * MLP_OUT];
};

__device__ __forceinline__ void load_weights( MlpSmem& s, const __nv_bfloat16* wbf, const float* master,
											  const float* norm )
{
	for ( int i = threadIdx.x; i < MLP_H * MLP_IN_PAD; i += blockDim.x )
		s.w1[i] = wbf[P_W1 + i];
	for ( int i = threadIdx.x; i < MLP_H * MLP_H; i += blockDim.x )
		s.w2[i] = wbf[P_W2 + i];
	for ( int i = threadIdx.x; i < MLP_OUT_PAD * MLP_H; i += blockDim.x )
		s.w3[i] = wbf[P_W3 + i];
	for ( int i = threadIdx.x; i < MLP_H; i += blockDim.x )
	{
		s.b1[i] = master[P_B1 + i];
		s.b2[i] = master[P_B2 + i];
	}
	for ( int i = threadIdx.x; i < MLP_OUT_PAD; i += blockDim.x )
		s.b3[i] = master[P_B3 + i];
	for ( int i = threadIdx.x; i < 2 * MLP_SAMPLE; i += blockDim.x )
		s.norm[i] = norm[i];
}

// Forward pass of the warp's 16 samples (features already in s.x[warp]);
// leaves the ReLU masks m1, m2 (z > 0), h1, h2 (BF16) and y (normalised
// outputs, FP32) in shared memory.
__device__ void warp_forward( MlpSmem& s, int warp, int lane )
{
	int g = lane >> 2, t = lane & 3;
	unsigned a[4], b[2];
	// layer 1: X [16x16] . W1^T [16x64]
	frag_a( a, s.x[warp], MLP_IN_PAD, 0, lane );
	for ( int n0 = 0; n0 < MLP_H; n0 += 8 )
	{
		float d[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
		frag_b_t( b, s.w1, MLP_IN_PAD, 0, n0, lane );
		mma16816( d, a, b );
		int c0 = n0 + 2 * t;
		float z[4] = { d[0] + s.b1[c0], d[1] + s.b1[c0 + 1], d[2] + s.b1[c0], d[3] + s.b1[c0 + 1] };
		int r[4] = { g, g, g + 8, g + 8 }, cc[4] = { c0, c0 + 1, c0, c0 + 1 };
		for ( int q = 0; q < 4; ++q )
		{
			s.m1[warp][r[q] * MLP_H + cc[q]] = z[q] > 0.0f ? 1 : 0;
			s.h1[warp][r[q] * MLP_H + cc[q]] = __float2bfloat16_rn( z[q] > 0.0f ? z[q] : 0.0f );
		}
	}
	__syncwarp();
	// layer 2: H1 [16x64] . W2^T [64x64]
	for ( int n0 = 0; n0 < MLP_H; n0 += 8 )
	{
		float d[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
		for ( int k0 = 0; k0 < MLP_H; k0 += 16 )
		{
			frag_a( a, s.h1[warp], MLP_H, k0, lane );
			frag_b_t( b, s.w2, MLP_H, k0, n0, lane );
			mma16816( d, a, b );
		}
		int c0 = n0 + 2 * t;
		float z[4] = { d[0] + s.b2[c0], d[1] + s.b2[c0 + 1], d[2] + s.b2[c0], d[3] + s.b2[c0 + 1] };
		int r[4] = { g, g, g + 8, g + 8 }, cc[4] = { c0, c0 + 1, c0, c0 + 1 };
		for ( int q = 0; q < 4; ++q )
		{
			s.m2[warp][r[q] * MLP_H + cc[q]] = z[q] > 0.0f ? 1 : 0;
			s.h2[warp][r[q] * MLP_H + cc[q]] = __float2bfloat16_rn( z[q] > 0.0f ? z[q] : 0.0f );
		}
	}
	__syncwarp();
	// layer 3: H2 [16x64] . W3^T [64x8]
	{
		float d[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
		for ( int k0 = 0; k0 < MLP_H; k0 += 16 )
		{
			frag_a( a, s.h2[warp], MLP_H, k0, lane );
			frag_b_t( b, s.w3, MLP_H, k0, 0, lane );
			mma16816( d, a, b );
		}
		int c0 = 2 * t;
		s.y[warp][g * MLP_OUT_PAD + c0] = d[0] + s.b3[c0];
		s.y[warp][g * MLP_OUT_PAD + c0 + 1] = d[1] + s.b3[c0 + 1];
		s.y[warp][( g + 8 ) * MLP_OUT_PAD + c0] = d[2] + s.b3[c0];
		s.y[warp][( g + 8 ) * MLP_OUT_PAD + c0 + 1] = d[3] + s.b3[c0 + 1];
	}
	__syncwarp();
}

// normalised BF16 features of one sample into row `row` of the warp tile
__device__ __forceinline__ void put_features( MlpSmem& s, int warp, int row, const float* f, bool valid )
{
	for ( int c = 0; c < MLP_IN_PAD; ++c )
	{
		float v = 0.0f;
		if ( valid && c < MLP_IN )
			v = ( f[c] - s.norm[c] ) * s.norm[MLP_SAMPLE + c];
		s.x[warp][row * MLP_IN_PAD + c] = __float2bfloat16_rn( v );
	}
}

// ---------------------------------------------------------------------------
// training: gradient of 0.5 * mean ||y - t||^2 over a batch
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__( MLP_THREADS )
	k_mlp_grad( const float* __restrict__ samples, const int* __restrict__ order, int first, int count,
				const __nv_bfloat16* __restrict__ wbf, const float* __restrict__ master,
				const float* __restrict__ norm, float* __restrict__ grad, float* __restrict__ loss )
{
	extern __shared__ __align__( 16 ) unsigned char mlpDyn[];
	MlpSmem& s = *reinterpret_cast<MlpSmem*>( mlpDyn );
	float* gacc = reinterpret_cast<float*>( mlpDyn + sizeof( MlpSmem ) );
	load_weights( s, wbf, master, norm );
	for ( int i = threadIdx.x; i < P_COUNT; i += blockDim.x )
		gacc[i] = 0.0f;
	__syncthreads();
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int g = lane >> 2, t = lane & 3;
	const float invB = 1.0f / (float)count;
	float lossAcc = 0.0f;
	const int tiles = ( count + 15 ) / 16;
	for ( int tile = blockIdx.x * MLP_WARPS + warp; tile < tiles; tile += gridDim.x * MLP_WARPS )
	{
		// 16 samples of this tile (lanes 0..15 fill one row each)
		if ( lane < 16 )
		{
			int i = tile * 16 + lane;
			bool valid = i < count;
			const float* smp = samples + (size_t)( valid ? order[first + i] : 0 ) * MLP_SAMPLE;
			put_features( s, warp, lane, smp, valid );
			for ( int o = 0; o < MLP_OUT; ++o )
				s.t[warp][lane * MLP_OUT + o] =
					valid ? ( smp[MLP_IN + o] - s.norm[MLP_IN + o] ) * s.norm[MLP_SAMPLE + MLP_IN + o] : 0.0f;
		}
		__syncwarp();
		warp_forward( s, warp, lane );
		// dy = (y - t) / B on valid rows; dz2 = (W3^T dy) * relu'(z2)
		float dy[16][MLP_OUT];
		for ( int r = 0; r < 16; ++r )
		{
			bool valid = tile * 16 + r < count;
			for ( int o = 0; o < MLP_OUT; ++o )
			{
				float e = valid ? s.y[warp][r * MLP_OUT_PAD + o] - s.t[warp][r * MLP_OUT + o] : 0.0f;
				dy[r][o] = e * invB;
				if ( lane == 0 )
					lossAcc += 0.5f * e * e;
			}
		}
		// db3, dW3 (2 x 64): lane owns hidden columns lane and lane + 32
		for ( int o = 0; o < MLP_OUT; ++o )
		{
			for ( int jj = 0; jj < 2; ++jj )
			{
				int j = lane + 32 * jj;
				float acc = 0.0f;
				for ( int r = 0; r < 16; ++r )
					acc += dy[r][o] * __bfloat162float( s.h2[warp][r * MLP_H + j] );
				atomicAdd( gacc + P_W3 + o * MLP_H + j, acc );
			}
			if ( lane == 0 )
			{
				float acc = 0.0f;
				for ( int r = 0; r < 16; ++r )
					acc += dy[r][o];
				atomicAdd( gacc + P_B3 + o, acc );
			}
		}
		// dz2 [16 x 64]
		for ( int jj = 0; jj < 2; ++jj )
		{
			int j = lane + 32 * jj;
			float w30 = __bfloat162float( s.w3[0 * MLP_H + j] ), w31 = __bfloat162float( s.w3[1 * MLP_H + j] );
			float db = 0.0f;
			for ( int r = 0; r < 16; ++r )
			{
				float dh = dy[r][0] * w30 + dy[r][1] * w31;
				float dz = s.m2[warp][r * MLP_H + j] ? dh : 0.0f;
				db += dz;
				s.dz[warp][r * MLP_H + j] = __float2bfloat16_rn( dz );
			}
			atomicAdd( gacc + P_B2 + j, db );
		}
		__syncwarp();
		unsigned a[4], b[2];
		// dW2 [64 x 64] += dz2^T [64 x 16] . H1 [16 x 64]
		for ( int m0 = 0; m0 < MLP_H; m0 += 16 )
		{
			frag_a_t( a, s.dz[warp], MLP_H, m0, lane );
			for ( int n0 = 0; n0 < MLP_H; n0 += 8 )
			{
				float d[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
				frag_b( b, s.h1[warp], MLP_H, 0, n0, lane );
				mma16816( d, a, b );
				int c0 = n0 + 2 * t;
				atomicAdd( gacc + P_W2 + ( m0 + g ) * MLP_H + c0, d[0] );
				atomicAdd( gacc + P_W2 + ( m0 + g ) * MLP_H + c0 + 1, d[1] );
				atomicAdd( gacc + P_W2 + ( m0 + g + 8 ) * MLP_H + c0, d[2] );
				atomicAdd( gacc + P_W2 + ( m0 + g + 8 ) * MLP_H + c0 + 1, d[3] );
			}
		}
		// dh1 [16 x 64] = dz2 [16 x 64] . W2 [64 x 64]; dz1 = dh1 * relu'(z1)
		float dz1v[8][4];
		for ( int n0 = 0, q = 0; n0 < MLP_H; n0 += 8, ++q )
		{
			float d[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
			for ( int k0 = 0; k0 < MLP_H; k0 += 16 )
			{
				frag_a( a, s.dz[warp], MLP_H, k0, lane );
				frag_b( b, s.w2, MLP_H, k0, n0, lane );
				mma16816( d, a, b );
			}
			int c0 = n0 + 2 * t;
			dz1v[q][0] = s.m1[warp][g * MLP_H + c0] ? d[0] : 0.0f;
			dz1v[q][1] = s.m1[warp][g * MLP_H + c0 + 1] ? d[1] : 0.0f;
			dz1v[q][2] = s.m1[warp][( g + 8 ) * MLP_H + c0] ? d[2] : 0.0f;
			dz1v[q][3] = s.m1[warp][( g + 8 ) * MLP_H + c0 + 1] ? d[3] : 0.0f;
		}
		__syncwarp();
		for ( int n0 = 0, q = 0; n0 < MLP_H; n0 += 8, ++q )
		{
			int c0 = n0 + 2 * t;
			s.dz[warp][g * MLP_H + c0] = __float2bfloat16_rn( dz1v[q][0] );
			s.dz[warp][g * MLP_H + c0 + 1] = __float2bfloat16_rn( dz1v[q][1] );
			s.dz[warp][( g + 8 ) * MLP_H + c0] = __float2bfloat16_rn( dz1v[q][2] );
			s.dz[warp][( g + 8 ) * MLP_H + c0 + 1] = __float2bfloat16_rn( dz1v[q][3] );
			atomicAdd( gacc + P_B1 + c0, dz1v[q][0] + dz1v[q][2] );
			atomicAdd( gacc + P_B1 + c0 + 1, dz1v[q][1] + dz1v[q][3] );
		}
		__syncwarp();
		// dW1 [64 x 16] += dz1^T [64 x 16] . X [16 x 16]
		for ( int m0 = 0; m0 < MLP_H; m0 += 16 )
		{
			frag_a_t( a, s.dz[warp], MLP_H, m0, lane );
			for ( int n0 = 0; n0 < MLP_IN_PAD; n0 += 8 )
			{
				float d[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
				frag_b( b, s.x[warp], MLP_IN_PAD, 0, n0, lane );
				mma16816( d, a, b );
				int c0 = n0 + 2 * t;
				atomicAdd( gacc + P_W1 + ( m0 + g ) * MLP_IN_PAD + c0, d[0] );
				atomicAdd( gacc + P_W1 + ( m0 + g ) * MLP_IN_PAD + c0 + 1, d[1] );
				atomicAdd( gacc + P_W1 + ( m0 + g + 8 ) * MLP_IN_PAD + c0, d[2] );
				atomicAdd( gacc + P_W1 + ( m0 + g + 8 ) * MLP_IN_PAD + c0 + 1, d[3] );
			}
		}
		__syncwarp();
	}
	__syncthreads();
	for ( int i = threadIdx.x; i < P_COUNT; i += blockDim.x )
		if ( gacc[i] != 0.0f )
			atomicAdd( grad + i, gacc[i] );
	if ( lane == 0 && lossAcc != 0.0f )
		atomicAdd( loss, lossAcc );
}

// padding entries (W1 columns 12..15, W3 rows 2..7, b3 entries 2..7) stay 0
__device__ __forceinline__ bool is_padding( int i )
{
	if ( i < P_W2 )
		return ( ( i - P_W1 ) % MLP_IN_PAD ) >= MLP_IN;
	if ( i >= P_W3 && i < P_B1 )
		return ( i - P_W3 ) / MLP_H >= MLP_OUT;
	if ( i >= P_B3 )
		return i - P_B3 >= MLP_OUT;
	return false;
}

__global__ void k_mlp_adam( float* master, __nv_bfloat16* wbf, float* grad, float* m, float* v, float lr, float b1t,
							float b2t )
{
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < P_COUNT; i += gridDim.x * blockDim.x )
	{
		float gi = is_padding( i ) ? 0.0f : grad[i];
		float mi = 0.9f * m[i] + 0.1f * gi;
		float vi = 0.999f * v[i] + 0.001f * gi * gi;
		m[i] = mi;
		v[i] = vi;
		float mh = mi / ( 1.0f - b1t ), vh = vi / ( 1.0f - b2t );
		float p = is_padding( i ) ? 0.0f : master[i] - lr * mh / ( sqrtf( vh ) + 1e-8f );
		master[i] = p;
		if ( i < P_B1 )
			wbf[i] = __float2bfloat16_rn( p );
		grad[i] = 0.0f;
	}
}

__global__ void k_mlp_refresh_bf16( const float* master, __nv_bfloat16* wbf )
{
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < P_B1; i += gridDim.x * blockDim.x )
		wbf[i] = __float2bfloat16_rn( master[i] );
}

// ---------------------------------------------------------------------------
// inference: predicted impulses of raw feature rows (12 floats per row)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void predict_tiles( MlpSmem& s, const float* feats, int count, float* out2 )
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int tiles = ( count + 15 ) / 16;
	for ( int tile = blockIdx.x * MLP_WARPS + warp; tile < tiles; tile += gridDim.x * MLP_WARPS )
	{
		if ( lane < 16 )
		{
			int i = tile * 16 + lane;
			put_features( s, warp, lane, feats + (size_t)( i < count ? i : 0 ) * MLP_IN, i < count );
		}
		__syncwarp();
		warp_forward( s, warp, lane );
		if ( lane < 16 )
		{
			int i = tile * 16 + lane;
			if ( i < count )
				for ( int o = 0; o < MLP_OUT; ++o )
					out2[(size_t)i * MLP_OUT + o] = s.y[warp][lane * MLP_OUT_PAD + o] *
														( 1.0f / s.norm[MLP_SAMPLE + MLP_IN + o] ) +
													s.norm[MLP_IN + o];
		}
		__syncwarp();
	}
}

__global__ void __launch_bounds__( MLP_THREADS ) k_mlp_predict( const float* feats, int count,
																const __nv_bfloat16* wbf, const float* master,
																const float* norm, float* out2 )
{
	extern __shared__ __align__( 16 ) unsigned char mlpDyn[];
	MlpSmem& s = *reinterpret_cast<MlpSmem*>( mlpDyn );
	load_weights( s, wbf, master, norm );
	__syncthreads();
	predict_tiles( s, feats, count, out2 );
}

// Warm start of the world step: the new manifold points the prepare stage
// listed get the predicted impulses (normal >= 0, friction cone) in place of
// zero; cached impulses of persisting points are untouched.
__global__ void __launch_bounds__( MLP_THREADS ) k_mlp_warm_start( DWorld w, const __nv_bfloat16* wbf,
																   const float* master, const float* norm )
{
	extern __shared__ __align__( 16 ) unsigned char mlpDyn[];
	MlpSmem& s = *reinterpret_cast<MlpSmem*>( mlpDyn );
	load_weights( s, wbf, master, norm );
	__syncthreads();
	int count = min( w.sc->newPointCount, w.newPointCap );
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int tiles = ( count + 15 ) / 16;
	for ( int tile = blockIdx.x * MLP_WARPS + warp; tile < tiles; tile += gridDim.x * MLP_WARPS )
	{
		if ( lane < 16 )
		{
			int i = tile * 16 + lane;
			put_features( s, warp, lane, w.newFeat + (size_t)( i < count ? i : 0 ) * MLP_IN, i < count );
		}
		__syncwarp();
		warp_forward( s, warp, lane );
		if ( lane < 16 )
		{
			int i = tile * 16 + lane;
			if ( i < count )
			{
				float ni = s.y[warp][lane * MLP_OUT_PAD + 0] * ( 1.0f / s.norm[MLP_SAMPLE + MLP_IN + 0] ) +
						   s.norm[MLP_IN + 0];
				float ti = s.y[warp][lane * MLP_OUT_PAD + 1] * ( 1.0f / s.norm[MLP_SAMPLE + MLP_IN + 1] ) +
						   s.norm[MLP_IN + 1];
				int2 kj = w.newPoint[i];
				float friction = w.newFeat[(size_t)i * MLP_IN + 11];
				ni = fmaxf( ni, 0.0f );
				ti = fminf( fmaxf( ti, -friction * ni ), friction * ni );
				float4 imp = w.kImp[kj.x];
				if ( kj.y == 0 )
				{
					imp.x = ni;
					imp.z = ti;
				}
				else
				{
					imp.y = ni;
					imp.w = ti;
				}
				w.kImp[kj.x] = imp;
			}
		}
		__syncwarp();
	}
}

// Training samples: features of each new point and the impulses the step
// ended with (written into the manifold by the solver's store stage).
__global__ void k_record_samples( DWorld w )
{
	int count = min( w.sc->newPointCount, w.newPointCap );
	for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x )
	{
		int slot = atomicAdd( &w.sc->sampleCount, 1 );
		if ( slot >= w.sampleCap )
			return;
		int2 kj = w.newPoint[i];
		int c = w.slotContact[kj.x];
		float4 im = w.mpI[2 * c + kj.y];
		float* o = w.samples + (size_t)slot * MLP_SAMPLE;
		for ( int f = 0; f < MLP_IN; ++f )
			o[f] = w.newFeat[(size_t)i * MLP_IN + f];
		o[MLP_IN] = im.x;
		o[MLP_IN + 1] = im.y;
	}
}

#define MLP_GRAD_SMEM ( sizeof( MlpSmem ) + sizeof( float ) * P_COUNT )

static void mlp_grad_setup()
{
	static bool done = false;
	if ( !done )
	{
		cudaFuncSetAttribute( k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MLP_GRAD_SMEM );
		cudaFuncSetAttribute( k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof( MlpSmem ) );
		cudaFuncSetAttribute( k_mlp_warm_start, cudaFuncAttributeMaxDynamicSharedMemorySize,
							  (int)sizeof( MlpSmem ) );
		done = true;
	}
}

void launch_learned_warm_start( DWorld& w, cudaStream_t st )
{
	if ( w.mlpModel < 0 || w.mlpModel >= MLP_MAX_MODELS || !s_models[w.mlpModel].used )
		return;
	MlpModel& M = s_models[w.mlpModel];
	k_mlp_warm_start<<<F2D_SMS, MLP_THREADS, sizeof( MlpSmem ), st>>>( w, M.wbf, M.master, M.norm );
}

void launch_record_samples( DWorld& w, cudaStream_t st )
{
	k_record_samples<<<grid_for( w.newPointCap ), 256, 0, st>>>( w );
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
static MlpModel* model_from( int32_t h )
{
	int i = h - 1;
	if ( i < 0 || i >= MLP_MAX_MODELS || !s_models[i].used )
		return nullptr;
	return s_models + i;
}

extern "C" F2D_API int32_t f2d_mlp_create( uint32_t seed )
{
	int slot = -1;
	for ( int i = 0; i < MLP_MAX_MODELS; ++i )
		if ( !s_models[i].used )
		{
			slot = i;
			break;
		}
	if ( slot < 0 )
		return 0;
	MlpModel& M = s_models[slot];
	memset( &M, 0, sizeof( M ) );
	if ( cudaMalloc( (void**)&M.master, sizeof( float ) * P_COUNT ) != cudaSuccess )
		return 0;
	cudaMalloc( (void**)&M.wbf, sizeof( __nv_bfloat16 ) * P_B1 );
	cudaMalloc( (void**)&M.grad, sizeof( float ) * P_COUNT );
	cudaMalloc( (void**)&M.m, sizeof( float ) * P_COUNT );
	cudaMalloc( (void**)&M.v, sizeof( float ) * P_COUNT );
	cudaMalloc( (void**)&M.norm, sizeof( float ) * 2 * MLP_SAMPLE );
	cudaMalloc( (void**)&M.loss, sizeof( float ) );
	// He-uniform initialisation from a 32-bit LCG, biases zero
	std::vector<float> p( P_COUNT, 0.0f );
	uint32_t x = seed * 2654435761u + 12345u;
	auto uni = [&]() {
		x = x * 1664525u + 1013904223u;
		return ( (float)( x >> 8 ) / 16777216.0f ) * 2.0f - 1.0f;
	};
	for ( int h = 0; h < MLP_H; ++h )
		for ( int c = 0; c < MLP_IN; ++c )
			p[P_W1 + h * MLP_IN_PAD + c] = uni() * sqrtf( 6.0f / MLP_IN );
	for ( int i = 0; i < MLP_H * MLP_H; ++i )
		p[P_W2 + i] = uni() * sqrtf( 6.0f / MLP_H );
	for ( int o = 0; o < MLP_OUT; ++o )
		for ( int j = 0; j < MLP_H; ++j )
			p[P_W3 + o * MLP_H + j] = uni() * sqrtf( 3.0f / MLP_H );
	cudaMemcpy( M.master, p.data(), sizeof( float ) * P_COUNT, cudaMemcpyHostToDevice );
	cudaMemset( M.grad, 0, sizeof( float ) * P_COUNT );
	cudaMemset( M.m, 0, sizeof( float ) * P_COUNT );
	cudaMemset( M.v, 0, sizeof( float ) * P_COUNT );
	std::vector<float> nrm( 2 * MLP_SAMPLE, 0.0f );
	for ( int i = 0; i < MLP_SAMPLE; ++i )
		nrm[MLP_SAMPLE + i] = 1.0f;
	cudaMemcpy( M.norm, nrm.data(), sizeof( float ) * nrm.size(), cudaMemcpyHostToDevice );
	k_mlp_refresh_bf16<<<8, 256>>>( M.master, M.wbf );
	cudaDeviceSynchronize();
	mlp_grad_setup();
	M.used = true;
	M.step = 0;
	return slot + 1;
}

extern "C" F2D_API void f2d_mlp_destroy( int32_t handle )
{
	MlpModel* M = model_from( handle );
	if ( M == nullptr )
		return;
	cudaDeviceSynchronize();
	cudaFree( M->master );
	cudaFree( M->wbf );
	cudaFree( M->grad );
	cudaFree( M->m );
	cudaFree( M->v );
	cudaFree( M->norm );
	cudaFree( M->loss );
	memset( M, 0, sizeof( *M ) );
}

extern "C" F2D_API int32_t f2d_mlp_param_count( void )
{
	return P_COUNT;
}

extern "C" F2D_API void f2d_mlp_get_params( int32_t handle, float* out )
{
	MlpModel* M = model_from( handle );
	if ( M )
		cudaMemcpy( out, M->master, sizeof( float ) * P_COUNT, cudaMemcpyDeviceToHost );
}

extern "C" F2D_API void f2d_mlp_set_params( int32_t handle, const float* in )
{
	MlpModel* M = model_from( handle );
	if ( M == nullptr )
		return;
	cudaMemcpy( M->master, in, sizeof( float ) * P_COUNT, cudaMemcpyHostToDevice );
	k_mlp_refresh_bf16<<<8, 256>>>( M->master, M->wbf );
	cudaDeviceSynchronize();
}

extern "C" F2D_API void f2d_mlp_set_normalization( int32_t handle, const float* mean14, const float* invStd14 )
{
	MlpModel* M = model_from( handle );
	if ( M == nullptr )
		return;
	cudaMemcpy( M->norm, mean14, sizeof( float ) * MLP_SAMPLE, cudaMemcpyHostToDevice );
	cudaMemcpy( M->norm + MLP_SAMPLE, invStd14, sizeof( float ) * MLP_SAMPLE, cudaMemcpyHostToDevice );
}

// Gradient of the batch loss 0.5 * mean ||y - t||^2 over all n samples
// (14 floats each) at the current parameters; no update. Returns the loss.
extern "C" F2D_API float f2d_mlp_gradient( int32_t handle, const float* samples14, int32_t n, float* grad )
{
	MlpModel* M = model_from( handle );
	if ( M == nullptr || n <= 0 )
		return 0.0f;
	float* ds = nullptr;
	int* ord = nullptr;
	cudaMalloc( (void**)&ds, sizeof( float ) * MLP_SAMPLE * (size_t)n );
	cudaMalloc( (void**)&ord, sizeof( int ) * (size_t)n );
	cudaMemcpy( ds, samples14, sizeof( float ) * MLP_SAMPLE * (size_t)n, cudaMemcpyHostToDevice );
	std::vector<int> o( n );
	for ( int i = 0; i < n; ++i )
		o[i] = i;
	cudaMemcpy( ord, o.data(), sizeof( int ) * (size_t)n, cudaMemcpyHostToDevice );
	cudaMemset( M->grad, 0, sizeof( float ) * P_COUNT );
	cudaMemset( M->loss, 0, sizeof( float ) );
	int tiles = ( n + 15 ) / 16;
	int blocks = ( tiles + MLP_WARPS - 1 ) / MLP_WARPS;
	if ( blocks > 4 * F2D_SMS )
		blocks = 4 * F2D_SMS;
	mlp_grad_setup();
	k_mlp_grad<<<blocks, MLP_THREADS, MLP_GRAD_SMEM>>>( ds, ord, 0, n, M->wbf, M->master, M->norm, M->grad, M->loss );
	float loss = 0.0f;
	cudaMemcpy( grad, M->grad, sizeof( float ) * P_COUNT, cudaMemcpyDeviceToHost );
	cudaMemcpy( &loss, M->loss, sizeof( float ), cudaMemcpyDeviceToHost );
	cudaMemset( M->grad, 0, sizeof( float ) * P_COUNT );
	cudaFree( ds );
	cudaFree( ord );
	return loss / (float)n;
}

// Adam training on the GPU: `epochs` passes over the n samples in shuffled
// batches of `batch`. Returns the mean loss of the last epoch.
extern "C" F2D_API float f2d_mlp_train( int32_t handle, const float* samples14, int32_t n, int32_t epochs,
										int32_t batch, float lr, uint32_t seed )
{
	MlpModel* M = model_from( handle );
	if ( M == nullptr || n <= 0 || batch <= 0 )
		return 0.0f;
	float* ds = nullptr;
	int* ord = nullptr;
	cudaMalloc( (void**)&ds, sizeof( float ) * MLP_SAMPLE * (size_t)n );
	cudaMalloc( (void**)&ord, sizeof( int ) * (size_t)n );
	cudaMemcpy( ds, samples14, sizeof( float ) * MLP_SAMPLE * (size_t)n, cudaMemcpyHostToDevice );
	std::vector<int> o( n );
	mlp_grad_setup();
	uint32_t x = seed * 747796405u + 2891336453u;
	float last = 0.0f;
	for ( int e = 0; e < epochs; ++e )
	{
		for ( int i = 0; i < n; ++i )
			o[i] = i;
		for ( int i = n - 1; i > 0; --i )
		{
			x = x * 1664525u + 1013904223u;
			int j = (int)( ( (uint64_t)x * (uint64_t)( i + 1 ) ) >> 32 );
			int tmp = o[i];
			o[i] = o[j];
			o[j] = tmp;
		}
		cudaMemcpy( ord, o.data(), sizeof( int ) * (size_t)n, cudaMemcpyHostToDevice );
		cudaMemset( M->loss, 0, sizeof( float ) );
		for ( int first = 0; first < n; first += batch )
		{
			int cnt = n - first < batch ? n - first : batch;
			int tiles = ( cnt + 15 ) / 16;
			int blocks = ( tiles + MLP_WARPS - 1 ) / MLP_WARPS;
			if ( blocks > 4 * F2D_SMS )
				blocks = 4 * F2D_SMS;
			k_mlp_grad<<<blocks, MLP_THREADS, MLP_GRAD_SMEM>>>( ds, ord, first, cnt, M->wbf, M->master, M->norm, M->grad,
																 M->loss );
			M->step += 1;
			float b1t = powf( 0.9f, (float)M->step ), b2t = powf( 0.999f, (float)M->step );
			k_mlp_adam<<<( P_COUNT + 255 ) / 256, 256>>>( M->master, M->wbf, M->grad, M->m, M->v, lr, b1t, b2t );
		}
		cudaMemcpy( &last, M->loss, sizeof( float ), cudaMemcpyDeviceToHost );
		last /= (float)n;
	}
	cudaFree( ds );
	cudaFree( ord );
	return last;
}

// Predicted (normal, tangent) impulses of n raw feature rows (12 floats).
extern "C" F2D_API void f2d_mlp_predict( int32_t handle, const float* feats12, int32_t n, float* out2 )
{
	MlpModel* M = model_from( handle );
	if ( M == nullptr || n <= 0 )
		return;
	float *df = nullptr, *dout = nullptr;
	cudaMalloc( (void**)&df, sizeof( float ) * MLP_IN * (size_t)n );
	cudaMalloc( (void**)&dout, sizeof( float ) * MLP_OUT * (size_t)n );
	cudaMemcpy( df, feats12, sizeof( float ) * MLP_IN * (size_t)n, cudaMemcpyHostToDevice );
	int tiles = ( n + 15 ) / 16;
	int blocks = ( tiles + MLP_WARPS - 1 ) / MLP_WARPS;
	if ( blocks > 4 * F2D_SMS )
		blocks = 4 * F2D_SMS;
	mlp_grad_setup();
	k_mlp_predict<<<blocks, MLP_THREADS, sizeof( MlpSmem )>>>( df, n, M->wbf, M->master, M->norm, dout );
	cudaMemcpy( out2, dout, sizeof( float ) * MLP_OUT * (size_t)n, cudaMemcpyDeviceToHost );
	cudaFree( df );
	cudaFree( dout );
}

bool f2d_internal_mlp_valid( int32_t handle )
{
	return model_from( handle ) != nullptr;
}
