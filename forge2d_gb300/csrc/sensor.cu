// Sensor overlaps and sensor events at the end of the step, as
// b2OverlapSensors (packages/forge2d/third_party/box2d/src/sensor.c:48-334,
// called at world.c:788-793).
//
// A sensor whose body is enabled and whose sensor events are on overlaps
// every other shape that has a proxy whose fat AABB meets the sensor's AABB
// (category against the sensor's mask, as the tree query), has sensor
// events on, sits on another body, passes the filter and is within
// 10 FLT_EPSILON by GJK with radii. One thread per visitor shape tests it
// against every sensor and appends (sensor index << 32 | shape) keys; the
// keys are sorted, and the begin events (keys new this step) and end events
// (keys gone) are compacted in key order, which is the order the reference
// emits them in: sensors in creation order, visitors by shape id.
#include "dtoi.cuh"
#include "dworld.cuh"
#include "dsort.cuh"
#include "kernels.cuh"

#define SENSOR_THREADS 256

// the sensor proxies of finalize.cu's continuous pass, restated for the
// distance query (shape.c:922-943)
__device__ __forceinline__ DProxy sensor_proxy( const float4* g, int type )
{
	DProxy p;
	float4 g0 = g[0], g1 = g[1];
	if ( type == ST_CIRCLE )
	{
		p.p[0] = mk( g0.x, g0.y );
		p.count = 1;
		p.radius = g1.x;
	}
	else if ( type == ST_POLYGON )
	{
		int count = __float_as_int( g1.y );
		for ( int i = 0; i < 4; ++i )
		{
			float4 v = g[2 + i];
			p.p[2 * i] = mk( v.x, v.y );
			p.p[2 * i + 1] = mk( v.z, v.w );
		}
		p.count = count;
		p.radius = g1.x;
	}
	else
	{
		p.p[0] = mk( g0.x, g0.y );
		p.p[1] = mk( g0.z, g0.w );
		p.count = 2;
		p.radius = type == ST_CAPSULE ? g1.x : 0.0f;
	}
	return p;
}

__device__ __forceinline__ fxf body_xf( const DWorld& w, int b )
{
	float4 x = w.xf[b];
	fxf t;
	t.p = mk( x.x, x.y );
	t.q.c = x.z;
	t.q.s = x.w;
	return t;
}

__global__ void __launch_bounds__( SENSOR_THREADS ) k_sensor_overlaps( DWorld w )
{
	const int S = w.sensorCount;
	for ( int o = blockIdx.x * blockDim.x + threadIdx.x; o < w.shapeCount; o += gridDim.x * blockDim.x )
	{
		int fo = w.sflags[o];
		if ( ( fo & ( SF_USED | SF_PROXY | SF_SENSOR_EVENTS ) ) != ( SF_USED | SF_PROXY | SF_SENSOR_EVENTS ) )
			continue;
		fbox fat = box_from4( w.fat[o] );
		int bo = w.shapeBody[o];
		unsigned long long catO = w.cat[o];
		for ( int k = 0; k < S; ++k )
		{
			int ss = w.sensorShapes[k];
			int fs = w.sflags[ss];
			int bs = w.shapeBody[ss];
			if ( ss == o || bs == bo || ( fs & SF_SENSOR_EVENTS ) == 0 || ( w.bflags[bs] & BF_ENABLED ) == 0 )
				continue;
			if ( ( catO & w.mask[ss] ) == 0ull || !box_overlaps( fat, box_from4( w.aabb[ss] ) ) )
				continue;
			// shape.c b2ShouldShapesCollide
			int ga = w.group[ss], gb = w.group[o];
			bool pass = ( ga == gb && ga != 0 ) ? ga > 0
											   : ( w.mask[ss] & catO ) != 0ull && ( w.cat[ss] & w.mask[o] ) != 0ull;
			if ( !pass )
				continue;
			DProxy pa = sensor_proxy( w.geom + (size_t)ss * GEOM_F4, shape_type( fs ) );
			DProxy pb = sensor_proxy( w.geom + (size_t)o * GEOM_F4, shape_type( fo ) );
			DCache cache;
			cache.count = 0;
			float d = gjk_distance( pa, pb, body_xf( w, bs ), body_xf( w, bo ), cache );
			// distance.c:592-603: radii applied past 0.1 linear slop
			if ( d > 0.1f * F2D_LINEAR_SLOP )
			{
				d = d - pa.radius - pb.radius;
				d = d > 0.0f ? d : 0.0f;
			}
			if ( d < 10.0f * FLT_EPSILON )
			{
				int slot = atomicAdd( &w.sc->sensorCur, 1 );
				if ( slot < w.sensorPairCap )
					w.sensorKeys[slot] = ( (unsigned long long)k << 32 ) | (unsigned)o;
				else
					atomicOr( &w.sc->error, ERR_EVENT_CAPACITY );
			}
		}
	}
}

__global__ void k_sensor_clamp( DWorld w )
{
	if ( w.sc->sensorCur > w.sensorPairCap )
		w.sc->sensorCur = w.sensorPairCap;
}

__device__ __forceinline__ bool key_in( const unsigned long long* keys, int n, unsigned long long key )
{
	int lo = 0, hi = n;
	while ( lo < hi )
	{
		int mid = ( lo + hi ) >> 1;
		if ( keys[mid] < key )
			lo = mid + 1;
		else
			hi = mid;
	}
	return lo < n && keys[lo] == key;
}

// one block: ordered compaction of the keys missing from the other list
__device__ void sensor_emit( const DWorld& w, const unsigned long long* keys, int n, const unsigned long long* other,
							 int nOther, int2* out, int* outCount )
{
	__shared__ int warpSums[SENSOR_THREADS / 32];
	__shared__ int base;
	if ( threadIdx.x == 0 )
		base = 0;
	__syncthreads();
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for ( int t = 0; t < n; t += SENSOR_THREADS )
	{
		int i = t + threadIdx.x;
		bool emit = i < n && !key_in( other, nOther, keys[i] );
		unsigned ballot = __ballot_sync( 0xffffffffu, emit );
		if ( lane == 0 )
			warpSums[wid] = __popc( ballot );
		__syncthreads();
		int before = 0, total = 0;
		for ( int k = 0; k < SENSOR_THREADS / 32; ++k )
		{
			before += k < wid ? warpSums[k] : 0;
			total += warpSums[k];
		}
		if ( emit )
		{
			int pos = base + before + __popc( ballot & ( ( 1u << lane ) - 1u ) );
			unsigned long long key = keys[i];
			out[pos] = make_int2( w.sensorShapes[(int)( key >> 32 )], (int)( key & 0xffffffffull ) );
		}
		__syncthreads();
		if ( threadIdx.x == 0 )
			base += total;
		__syncthreads();
	}
	if ( threadIdx.x == 0 )
		*outCount = base;
}

__global__ void __launch_bounds__( SENSOR_THREADS ) k_sensor_events( DWorld w )
{
	const int nCur = w.sc->sensorCur, nPrev = w.sc->sensorPrev;
	sensor_emit( w, w.sensorKeys, nCur, w.sensorPrevKeys, nPrev, w.sensorBeginEv, &w.sc->sensorBegin );
	sensor_emit( w, w.sensorPrevKeys, nPrev, w.sensorKeys, nCur, w.sensorEndEv, &w.sc->sensorEnd );
	__syncthreads();
	for ( int i = threadIdx.x; i < nCur; i += SENSOR_THREADS )
		w.sensorPrevKeys[i] = w.sensorKeys[i];
	if ( threadIdx.x == 0 )
	{
		w.sc->sensorPrev = nCur;
		w.sc->sensorCur = 0;
	}
}

void launch_sensors( DWorld& w, StepScratch& s, cudaStream_t st )
{
	if ( w.sensorCount == 0 )
		return;
	int grid = ( w.shapeCap + SENSOR_THREADS - 1 ) / SENSOR_THREADS;
	if ( grid > F2D_SMS * 8 )
		grid = F2D_SMS * 8;
	if ( grid < 1 )
		grid = 1;
	k_sensor_overlaps<<<grid, SENSOR_THREADS, 0, st>>>( w );
	k_sensor_clamp<<<1, 1, 0, st>>>( w );
	int bits = 32;
	while ( bits < 64 && ( 1ll << ( bits - 32 ) ) < w.sensorCount )
		bits += 1;
	// keys are unique, so their order alone fixes the result
	sort_coop<unsigned long long>( w.sensorKeys, nullptr, w.sensorKeysAlt, nullptr, &w.sc->sensorCur, bits,
								   w.sortHist, &w.sc->barrierCount, &w.sc->error, s.sortBlocks64, st );
	k_sensor_events<<<1, SENSOR_THREADS, 0, st>>>( w );
}
