// Contact state changes and constraint-graph colouring.
//
// Box2D v3.1.1 applies the step's contact state changes serially in contact
// id order (world.c:586-686): destroy disjoint contacts (freeing their ids
// LIFO), add contacts that began touching to the lowest graph colour whose
// body bitsets are free for both bodies, remove contacts that stopped
// touching (constraint_graph.c:68-212). The colour a contact receives depends
// on every earlier add and remove that touched one of its bodies.
//
// The serial result is reproduced exactly in parallel: ops are processed in
// rounds, and an op executes once it is the lowest-numbered pending op on
// each of its non-static bodies (per-body atomicMin locks). Ops executing in
// the same round therefore touch disjoint bodies and every op sees exactly
// the body colour masks the serial order would give it. The first round,
// which carries most ops, runs grid-wide; the ops it leaves pending go
// through the remaining rounds in one block. The order-dependent outputs
// (freed ids, events, flags, the overflow array) are then written in op
// order from prefix sums.
#include "dscan.cuh"
#include "dsort.cuh"
#include "dsync.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

#include <climits>

#define GRAPH_THREADS 1024
#define GRAPH_MAX_ROUNDS 100000
#define OVF_HASH 4096	  // shared-memory hash of overflow-array positions
#define OVF_LIST_SMEM 2048 // overflow-array length handled in shared memory

enum
{
	OP_NONE = 0,
	OP_ADD = 1,
	OP_REMOVE = 2
};

__device__ __forceinline__ int body_solver_index( const DWorld& w, int b )
{
	return body_type( w.bflags[b] ) == 0 ? -1 : b;
}

__device__ __forceinline__ int op_count( const DWorld& w )
{
	int n = w.sc->opCount;
	return n > w.opCap ? w.opCap : n;
}

// Graph kind of each op, its solver bodies, and the lock reset of the first
// round (world.c:586-686 order of cases).
__global__ void k_op_prepare( DWorld w, int* gkind )
{
	int nOps = op_count( w );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		int c = w.opContact[k];
		int kind = w.opKind[k];
		int f = w.cflags[c];
		int g = OP_NONE;
		if ( kind == 1 )
			g = OP_ADD;
		else if ( ( kind == 2 ) || ( kind == 0 && ( f & CF_TOUCHING ) ) )
			g = OP_REMOVE;
		w.opColor[k] = g == OP_REMOVE ? w.ccolor[c] : F2D_NULL;
		w.opDone[k] = g == OP_NONE ? 1 : 0;
		gkind[k] = g;
		int2 ab = make_int2( -1, -1 );
		if ( g != OP_NONE )
		{
			int2 bd = w.cbody[c];
			ab.x = body_solver_index( w, bd.x );
			ab.y = body_solver_index( w, bd.y );
			if ( ab.x >= 0 )
				w.colorLock[ab.x] = INT_MAX;
			if ( ab.y >= 0 )
				w.colorLock[ab.y] = INT_MAX;
		}
		w.opBodies[k] = ab;
	}
}

__global__ void k_op_lock( DWorld w )
{
	int nOps = op_count( w );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		if ( w.opDone[k] )
			continue;
		int2 ab = w.opBodies[k];
		if ( ab.x >= 0 )
			atomicMin( w.colorLock + ab.x, k );
		if ( ab.y >= 0 )
			atomicMin( w.colorLock + ab.y, k );
	}
}

// Add to the lowest colour free on both bodies (constraint_graph.c:68-140;
// no static contacts in colour 0), or clear the removed colour's bits
// (constraint_graph.c:184-212).
__device__ __forceinline__ void apply_op( const DWorld& w, int k, int g, int a, int b )
{
	if ( g == OP_ADD )
	{
		unsigned ma = a >= 0 ? __ldcg( w.colorMask + a ) : 0u;
		unsigned mb = b >= 0 ? __ldcg( w.colorMask + b ) : 0u;
		int color = F2D_OVERFLOW;
		if ( a >= 0 && b >= 0 )
		{
			unsigned used = ma | mb;
			for ( int i = 0; i < F2D_OVERFLOW; ++i )
				if ( ( used & ( 1u << i ) ) == 0 )
				{
					color = i;
					break;
				}
			if ( color != F2D_OVERFLOW )
			{
				w.colorMask[a] = ma | ( 1u << color );
				w.colorMask[b] = mb | ( 1u << color );
			}
		}
		else
		{
			int d = a >= 0 ? a : b;
			unsigned md = a >= 0 ? ma : mb;
			for ( int i = 1; i < F2D_OVERFLOW; ++i )
				if ( ( md & ( 1u << i ) ) == 0 )
				{
					color = i;
					break;
				}
			if ( color != F2D_OVERFLOW )
				w.colorMask[d] = md | ( 1u << color );
		}
		w.opColor[k] = color;
	}
	else
	{
		int color = w.opColor[k];
		if ( color >= 0 && color != F2D_OVERFLOW )
		{
			unsigned bit = 1u << color;
			if ( a >= 0 )
				w.colorMask[a] = __ldcg( w.colorMask + a ) & ~bit;
			if ( b >= 0 )
				w.colorMask[b] = __ldcg( w.colorMask + b ) & ~bit;
		}
	}
}

// First round, grid-wide: lock owners apply; the rest are flagged pending.
__global__ void k_op_round( DWorld w, const int* gkind, int* pending )
{
	int nOps = op_count( w );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
	{
		int pend = 0;
		if ( w.opDone[k] == 0 )
		{
			int2 ab = w.opBodies[k];
			bool own = ( ab.x < 0 || w.colorLock[ab.x] == k ) && ( ab.y < 0 || w.colorLock[ab.y] == k );
			if ( own )
				apply_op( w, k, gkind[k], ab.x, ab.y );
			else
				pend = 1;
		}
		pending[k] = pend;
	}
}

__global__ void k_op_pending_list( DWorld w, const int* pending, const int* pos, int* list )
{
	int nOps = op_count( w );
	for ( int k = blockIdx.x * blockDim.x + threadIdx.x; k < nOps; k += gridDim.x * blockDim.x )
		if ( pending[k] )
			list[pos[k]] = k;
}

// Remaining rounds in one block over the pending list, compacted in place
// after every round.
__global__ void __launch_bounds__( GRAPH_THREADS ) k_color_rounds( DWorld w, const int* gkind, int* list )
{
	__shared__ int smem[32];
	int n = w.sc->pendingOps;
	int round = 1;
	for ( ; n > 0 && round < GRAPH_MAX_ROUNDS; ++round )
	{
		for ( int i = threadIdx.x; i < n; i += blockDim.x )
		{
			int2 ab = w.opBodies[list[i]];
			if ( ab.x >= 0 )
				w.colorLock[ab.x] = INT_MAX;
			if ( ab.y >= 0 )
				w.colorLock[ab.y] = INT_MAX;
		}
		__syncthreads();
		for ( int i = threadIdx.x; i < n; i += blockDim.x )
		{
			int k = list[i];
			int2 ab = w.opBodies[k];
			if ( ab.x >= 0 )
				atomicMin( w.colorLock + ab.x, k );
			if ( ab.y >= 0 )
				atomicMin( w.colorLock + ab.y, k );
		}
		__syncthreads();
		int running = 0;
		for ( int base = 0; base < n; base += blockDim.x )
		{
			int i = base + threadIdx.x;
			int k = -1, keep = 0;
			if ( i < n )
			{
				k = list[i];
				int2 ab = w.opBodies[k];
				bool own = ( ab.x < 0 || __ldcg( w.colorLock + ab.x ) == k ) &&
						   ( ab.y < 0 || __ldcg( w.colorLock + ab.y ) == k );
				if ( own )
					apply_op( w, k, gkind[k], ab.x, ab.y );
				else
					keep = 1;
			}
			int total;
			int excl = block_exclusive_scan_1024( keep, smem, &total );
			if ( keep )
				list[running + excl] = k;
			running += total;
			__syncthreads();
		}
		n = running;
	}
	if ( threadIdx.x == 0 )
	{
		w.sc->colorRounds = round;
		if ( round >= GRAPH_MAX_ROUNDS )
			atomicOr( &w.sc->error, ERR_COLOR_ROUNDS );
	}
}

// One look-back chain of k_op_outputs: publish this tile's aggregate, sum
// the predecessors' values until an inclusive prefix is found, publish the
// inclusive prefix. Returns the exclusive prefix.
__device__ __forceinline__ int op_chain( unsigned long long* st, int tile, int aggregate, int* err )
{
	const unsigned long long AGG = 1ull, PREFIX = 2ull;
	if ( tile == 0 )
	{
		st_release_u64( st, ( PREFIX << 32 ) | (unsigned)aggregate );
		return 0;
	}
	st_release_u64( st + tile, ( AGG << 32 ) | (unsigned)aggregate );
	int prefix = 0;
	int j = tile - 1;
	long long spins = 0;
	while ( j >= 0 )
	{
		unsigned long long v = ld_acquire_u64( st + j );
		unsigned long long flag = v >> 32;
		if ( flag == 0ull )
		{
			if ( ++spins > F2D_SPIN_LIMIT )
			{
				atomicOr( err, ERR_BARRIER_TIMEOUT );
				break;
			}
			continue;
		}
		prefix += (int)(unsigned)( v & 0xffffffffull );
		if ( flag == PREFIX )
			break;
		j -= 1;
	}
	st_release_u64( st + tile, ( PREFIX << 32 ) | (unsigned)( prefix + aggregate ) );
	return prefix;
}

// Freed ids, begin/end events, contact flags and the list of overflow ops,
// all in op order (world.c:586-686). Tiles are claimed in launch order and
// chained by decoupled look-back.
__global__ void __launch_bounds__( OPS_TILE ) k_op_outputs( DWorld w, const int* gkind, int* ovOps, int serialGraph )
{
	__shared__ int smem[32];
	__shared__ int s_tile, s_prefix[OPS_SCAN_CHAINS];
	const int nOps = op_count( w );
	const int F = w.sc->contactFreeCount;
	if ( threadIdx.x == 0 )
		s_tile = (int)atomicAdd( (unsigned*)w.opScan, 1u );
	__syncthreads();
	const int tile = s_tile;
	const int base = tile * OPS_TILE;
	if ( base >= nOps )
	{
		if ( tile == 0 && threadIdx.x == 0 )
		{
			w.sc->beginCount = 0;
			w.sc->endCount = 0;
			w.sc->overflowOps = 0;
		}
		return;
	}
	const int k = base + threadIdx.x;
	int isFree = 0, isBegin = 0, isEnd = 0, isOvf = 0;
	int c = -1, kind = -1, f = 0;
	if ( k < nOps )
	{
		c = w.opContact[k];
		kind = w.opKind[k];
		f = w.cflags[c];
		isFree = kind == 0;
		isBegin = kind == 1 && ( f & CF_EVENTS );
		isEnd = ( kind == 2 || ( kind == 0 && ( f & CF_TOUCHING ) ) ) && ( f & CF_EVENTS );
		// the serial island path maintains the overflow array itself
		bool serial = serialGraph || ( w.isl && w.isl->serialOps );
		isOvf = !serial && gkind[k] != OP_NONE && w.opColor[k] == F2D_OVERFLOW;
	}
	// per-tile counts stay below 2^16: two counters per scanned int
	int t01, t23;
	int e01 = block_exclusive_scan_1024( isFree | ( isBegin << 16 ), smem, &t01 );
	int e23 = block_exclusive_scan_1024( isEnd | ( isOvf << 16 ), smem, &t23 );
	if ( threadIdx.x < OPS_SCAN_CHAINS )
	{
		int agg = threadIdx.x == 0 ? ( t01 & 0xffff ) : threadIdx.x == 1 ? ( t01 >> 16 )
												   : threadIdx.x == 2 ? ( t23 & 0xffff )
																	  : ( t23 >> 16 );
		int tiles = ( w.opCap + OPS_TILE - 1 ) / OPS_TILE + 1;
		unsigned long long* st = w.opScan + 1 + (size_t)threadIdx.x * tiles;
		s_prefix[threadIdx.x] = op_chain( st, tile, agg, &w.sc->error );
	}
	__syncthreads();
	if ( k < nOps )
	{
		int2 sh = w.cshape[c];
		if ( isBegin )
		{
			int e = s_prefix[1] + ( e01 >> 16 );
			if ( e < w.eventCap )
			{
				w.beginEv[2 * e] = sh.x;
				w.beginEv[2 * e + 1] = sh.y;
				// world.c:630-640: the event carries this step's manifold
				float4 mn = w.mnorm[c];
				int count = __float_as_int( mn.w );
				float* o = w.beginEvF + 9 * (size_t)e;
				o[0] = mn.x;
				o[1] = mn.y;
				o[2] = (float)count;
				for ( int k = 0; k < 2; ++k )
				{
					float4 pb = w.mpB[2 * c + k];
					o[3 + 3 * k] = k < count ? pb.x : 0.0f;
					o[4 + 3 * k] = k < count ? pb.y : 0.0f;
					o[5 + 3 * k] = k < count ? pb.z : 0.0f;
				}
			}
		}
		if ( isEnd )
		{
			int e = s_prefix[2] + ( e23 & 0xffff );
			if ( e < w.eventCap )
			{
				w.endEv[2 * e] = sh.x;
				w.endEv[2 * e + 1] = sh.y;
			}
		}
		if ( isOvf )
			ovOps[s_prefix[3] + ( e23 >> 16 )] = k;
		if ( kind == 0 )
		{
			w.contactFree[F + s_prefix[0] + ( e01 & 0xffff )] = c;
			w.cflags[c] = 0;
			w.ccolor[c] = F2D_NULL;
		}
		else if ( kind == 1 )
		{
			w.cflags[c] = ( f | CF_TOUCHING ) & ~CF_STARTED;
			w.ccolor[c] = w.opColor[k];
		}
		else
		{
			w.cflags[c] = f & ~( CF_TOUCHING | CF_STOPPED );
			w.ccolor[c] = F2D_NULL;
		}
	}
	if ( base + OPS_TILE >= nOps && threadIdx.x == 0 )
	{
		// last tile: totals (every other tile has read F and nOps by now, as
		// its aggregate is part of this tile's prefix)
		int totFree = s_prefix[0] + ( t01 & 0xffff );
		int totBegin = s_prefix[1] + ( t01 >> 16 );
		int totEnd = s_prefix[2] + ( t23 & 0xffff );
		w.sc->contactFreeCount = F + totFree;
		w.sc->beginCount = min( totBegin, w.eventCap );
		w.sc->endCount = min( totEnd, w.eventCap );
		w.sc->overflowOps = s_prefix[3] + ( t23 >> 16 );
		if ( totBegin > w.eventCap || totEnd > w.eventCap )
			atomicOr( &w.sc->error, ERR_EVENT_CAPACITY );
	}
}

// Overflow-array maintenance in op order: append, or swap-remove
// (constraint_graph.c:140-212 on the overflow colour). One thread applies
// the ops on a shared-memory copy of the array with a hash of positions;
// arrays too long for shared memory take the same steps in global memory.
__global__ void __launch_bounds__( GRAPH_THREADS ) k_overflow_ops( DWorld w, const int* gkind, const int* ovOps )
{
	__shared__ int sList[OVF_LIST_SMEM];
	__shared__ int sKey[OVF_HASH];
	__shared__ int sPos[OVF_HASH];
	__shared__ int sCount;
	const int nov = w.sc->overflowOps;
	int count = w.sc->overflowCount;
	if ( threadIdx.x == 0 )
		w.sc->opCount = 0;
	if ( nov == 0 )
		return;
	if ( count + nov > OVF_LIST_SMEM )
	{
		if ( threadIdx.x == 0 )
		{
			for ( int i = 0; i < nov; ++i )
			{
				int k = ovOps[i];
				int c = w.opContact[k];
				if ( gkind[k] == OP_ADD )
				{
					w.overflowList[count] = c;
					w.coverflowIndex[c] = count;
					count += 1;
				}
				else
				{
					int idx = w.coverflowIndex[c];
					int last = count - 1;
					if ( idx >= 0 && idx <= last )
					{
						if ( idx != last )
						{
							int moved = w.overflowList[last];
							w.overflowList[idx] = moved;
							w.coverflowIndex[moved] = idx;
						}
						count -= 1;
					}
					w.coverflowIndex[c] = F2D_NULL;
				}
			}
			w.sc->overflowCount = count;
		}
		return;
	}
	for ( int i = threadIdx.x; i < OVF_HASH; i += blockDim.x )
		sKey[i] = -1;
	__syncthreads();
	// positions of the current entries (contact ids are unique in the array)
	for ( int i = threadIdx.x; i < count; i += blockDim.x )
	{
		int c = w.overflowList[i];
		sList[i] = c;
		unsigned h = ( (unsigned)c * 2654435761u ) & ( OVF_HASH - 1 );
		for ( int probe = 0; probe < OVF_HASH; ++probe )
		{
			if ( atomicCAS( sKey + h, -1, c ) == -1 )
			{
				sPos[h] = i;
				break;
			}
			h = ( h + 1 ) & ( OVF_HASH - 1 );
		}
	}
	__syncthreads();
	if ( threadIdx.x == 0 )
	{
		for ( int i = 0; i < nov; ++i )
		{
			int k = ovOps[i];
			int c = w.opContact[k];
			unsigned h = ( (unsigned)c * 2654435761u ) & ( OVF_HASH - 1 );
			int probe = 0;
			while ( probe < OVF_HASH && sKey[h] != c && sKey[h] != -1 )
			{
				h = ( h + 1 ) & ( OVF_HASH - 1 );
				++probe;
			}
			bool found = probe < OVF_HASH && sKey[h] == c;
			if ( gkind[k] == OP_ADD )
			{
				sList[count] = c;
				if ( !found && probe < OVF_HASH )
					sKey[h] = c;
				if ( probe < OVF_HASH )
					sPos[h] = count;
				count += 1;
			}
			else if ( found )
			{
				int idx = sPos[h];
				int last = count - 1;
				// the entry stays as a tombstone with an out-of-range position
				sPos[h] = -1;
				if ( idx >= 0 && idx <= last )
				{
					if ( idx != last )
					{
						int moved = sList[last];
						sList[idx] = moved;
						unsigned hm = ( (unsigned)moved * 2654435761u ) & ( OVF_HASH - 1 );
						for ( int pm = 0; pm < OVF_HASH && sKey[hm] != moved; ++pm )
							hm = ( hm + 1 ) & ( OVF_HASH - 1 );
						if ( sKey[hm] == moved )
							sPos[hm] = idx;
					}
					count -= 1;
				}
			}
			w.coverflowIndex[c] = F2D_NULL;
		}
		w.sc->overflowCount = count;
		sCount = count;
	}
	__syncthreads();
	count = sCount;
	for ( int i = threadIdx.x; i < count; i += blockDim.x )
	{
		int c = sList[i];
		w.overflowList[i] = c;
		w.coverflowIndex[c] = i;
	}
}

// Joint colours are assigned when joints are created (constraint_graph.c:
// 214-267; joints may take colour 0 even against a static body). Joints
// created since the last step are coloured here, in creation order.
__global__ void k_joint_ops( DWorld w, int count )
{
	if ( blockIdx.x != 0 || threadIdx.x != 0 )
		return;
	for ( int i = 0; i < count; ++i )
	{
		int j = w.pendingJointOps[i];
		int2 jb = w.jbody[j];
		int a = body_solver_index( w, jb.x ), b = body_solver_index( w, jb.y );
		int color = F2D_OVERFLOW;
		if ( a >= 0 && b >= 0 )
		{
			unsigned used = w.colorMask[a] | w.colorMask[b];
			for ( int c = 0; c < F2D_OVERFLOW; ++c )
				if ( ( used & ( 1u << c ) ) == 0 )
				{
					color = c;
					break;
				}
			if ( color != F2D_OVERFLOW )
			{
				w.colorMask[a] |= 1u << color;
				w.colorMask[b] |= 1u << color;
			}
		}
		else if ( a >= 0 || b >= 0 )
		{
			int d = a >= 0 ? a : b;
			for ( int c = 0; c < F2D_OVERFLOW; ++c )
				if ( ( w.colorMask[d] & ( 1u << c ) ) == 0 )
				{
					color = c;
					break;
				}
			if ( color != F2D_OVERFLOW )
				w.colorMask[d] |= 1u << color;
		}
		w.jcolor[j] = color;
		w.jcolorSet[j] = color == F2D_OVERFLOW ? 0 : ( a >= 0 ? 1 : 0 ) | ( b >= 0 ? 2 : 0 );
		if ( color == F2D_OVERFLOW )
		{
			w.overflowJoints[w.sc->overflowJointCount] = j;
			w.sc->overflowJointCount += 1;
		}
	}
}

void launch_graph( DWorld& w, StepScratch& s, cudaStream_t st )
{
	const size_t cap = (size_t)w.opCap;
	int* gkind = s.tmpA;
	int* pending = s.tmpA + cap;
	int* pos = s.tmpB;
	int* list = s.tmpB + cap;
	int* ovOps = s.tmpA + cap; // reuses the pending flags once the rounds are done
	int g = grid_for( w.opCap );
	k_op_prepare<<<g, 256, 0, st>>>( w, gkind );
	// sleeping worlds: island links and unlinks (island.cu); a step whose
	// changes wake a sleeping set applies them serially there, colours
	// included, and leaves no op for the rounds below
	if ( w.isl )
		launch_isl_ops( w, s, st, gkind );
	k_op_lock<<<g, 256, 0, st>>>( w );
	k_op_round<<<g, 256, 0, st>>>( w, gkind, pending );
	scan_lookback( pending, pos, &w.sc->opCount, 0, w.opCap, &w.sc->pendingOps, s.scanState, &w.sc->error, st );
	k_op_pending_list<<<g, 256, 0, st>>>( w, pending, pos, list );
	k_color_rounds<<<1, GRAPH_THREADS, 0, st>>>( w, gkind, list );
	cudaMemsetAsync( w.opScan, 0, sizeof( unsigned long long ) * (size_t)OPS_SCAN_WORDS( w.opCap ), st );
	k_op_outputs<<<( w.opCap + OPS_TILE - 1 ) / OPS_TILE, OPS_TILE, 0, st>>>( w, gkind, ovOps, 0 );
	k_overflow_ops<<<1, GRAPH_THREADS, 0, st>>>( w, gkind, ovOps );
}

void launch_joint_ops( DWorld& w, cudaStream_t st )
{
	if ( w.pendingJointCount > 0 )
		k_joint_ops<<<1, 1, 0, st>>>( w, w.pendingJointCount );
}
