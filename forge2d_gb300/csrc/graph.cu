// Contact state changes and constraint-graph colouring.
//
// Box2D v3.1.1 applies the step's contact state changes serially in contact
// id order (world.c:586-686): destroy disjoint contacts (freeing their ids
// LIFO), add contacts that began touching to the lowest graph colour whose
// body bitsets are free for both bodies, remove contacts that stopped
// touching (constraint_graph.c:68-212). The colour a contact receives depends
// on every earlier add and remove that touched one of its bodies.
//
// This kernel reproduces that serial result exactly in parallel: ops are
// processed in rounds, and an op executes once it is the lowest-numbered
// pending op on each of its non-static bodies (per-body atomicMin locks).
// Ops executing in the same round therefore touch disjoint bodies and every
// op sees exactly the body colour masks the serial order would give it.
#include "dscan.cuh"
#include "dworld.cuh"
#include "kernels.cuh"

#include <climits>

#define GRAPH_THREADS 1024
#define GRAPH_MAX_ROUNDS 100000

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

__device__ __forceinline__ int chunk_scan( int v, int* smem, int* total )
{
	return block_exclusive_scan_1024( v, smem, total );
}

__global__ void __launch_bounds__( GRAPH_THREADS ) k_color_ops( DWorld w, int* scratch )
{
	__shared__ int smem[32];
	__shared__ int s_pending;
	int nOps = w.sc->opCount;
	if ( nOps > w.opCap )
		nOps = w.opCap;

	// classify: opDone = 1 for ops that do not touch the graph
	for ( int k = threadIdx.x; k < nOps; k += blockDim.x )
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
		scratch[k] = g;
	}
	__syncthreads();

	int round = 0;
	for ( ; round < GRAPH_MAX_ROUNDS; ++round )
	{
		if ( threadIdx.x == 0 )
			s_pending = 0;
		// reset locks of bodies touched by pending ops
		for ( int k = threadIdx.x; k < nOps; k += blockDim.x )
		{
			if ( w.opDone[k] )
				continue;
			int2 bd = w.cbody[w.opContact[k]];
			int a = body_solver_index( w, bd.x ), b = body_solver_index( w, bd.y );
			if ( a >= 0 )
				w.colorLock[a] = INT_MAX;
			if ( b >= 0 )
				w.colorLock[b] = INT_MAX;
		}
		__syncthreads();
		for ( int k = threadIdx.x; k < nOps; k += blockDim.x )
		{
			if ( w.opDone[k] )
				continue;
			int2 bd = w.cbody[w.opContact[k]];
			int a = body_solver_index( w, bd.x ), b = body_solver_index( w, bd.y );
			if ( a >= 0 )
				atomicMin( w.colorLock + a, k );
			if ( b >= 0 )
				atomicMin( w.colorLock + b, k );
		}
		__syncthreads();
		int localPending = 0;
		for ( int k = threadIdx.x; k < nOps; k += blockDim.x )
		{
			if ( w.opDone[k] )
				continue;
			int2 bd = w.cbody[w.opContact[k]];
			int a = body_solver_index( w, bd.x ), b = body_solver_index( w, bd.y );
			bool own = ( a < 0 || w.colorLock[a] == k ) && ( b < 0 || w.colorLock[b] == k );
			if ( !own )
			{
				localPending += 1;
				continue;
			}
			if ( scratch[k] == OP_ADD )
			{
				unsigned ma = a >= 0 ? w.colorMask[a] : 0u;
				unsigned mb = b >= 0 ? w.colorMask[b] : 0u;
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
					// no static contacts in colour 0 (constraint_graph.c:105-135)
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
						w.colorMask[a] &= ~bit;
					if ( b >= 0 )
						w.colorMask[b] &= ~bit;
				}
			}
			w.opDone[k] = 1;
		}
		if ( localPending )
			atomicAdd( &s_pending, localPending );
		__syncthreads();
		if ( s_pending == 0 )
			break;
		__syncthreads();
	}
	if ( threadIdx.x == 0 )
	{
		w.sc->colorRounds = round + 1;
		if ( round >= GRAPH_MAX_ROUNDS )
			atomicOr( &w.sc->error, ERR_COLOR_ROUNDS );
	}
	__syncthreads();

	// overflow-array maintenance in op order (append / swap-remove): compact
	// the ops that involve the overflow colour, then apply them serially
	int running = 0;
	int* ovList = scratch + w.opCap;
	for ( int base = 0; base < nOps; base += blockDim.x )
	{
		int k = base + threadIdx.x;
		int v = 0;
		if ( k < nOps && scratch[k] != OP_NONE && w.opColor[k] == F2D_OVERFLOW )
			v = 1;
		int total;
		int excl = chunk_scan( v, smem, &total );
		if ( v )
			ovList[running + excl] = k;
		running += total;
		__syncthreads();
	}
	if ( threadIdx.x == 0 )
	{
		int count = w.sc->overflowCount;
		for ( int i = 0; i < running; ++i )
		{
			int k = ovList[i];
			int c = w.opContact[k];
			if ( scratch[k] == OP_ADD )
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
	__syncthreads();

	// free list, events and contact flag updates, all in op order
	int F = w.sc->contactFreeCount;
	int runFree = 0, runBegin = 0, runEnd = 0;
	for ( int base = 0; base < nOps; base += blockDim.x )
	{
		int k = base + threadIdx.x;
		int isFree = 0, isBegin = 0, isEnd = 0;
		int c = -1, kind = -1, f = 0;
		if ( k < nOps )
		{
			c = w.opContact[k];
			kind = w.opKind[k];
			f = w.cflags[c];
			isFree = kind == 0;
			isBegin = kind == 1 && ( f & CF_EVENTS );
			isEnd = ( kind == 2 || ( kind == 0 && ( f & CF_TOUCHING ) ) ) && ( f & CF_EVENTS );
		}
		int tFree, tBegin, tEnd;
		int eFree = chunk_scan( isFree, smem, &tFree );
		int eBegin = chunk_scan( isBegin, smem, &tBegin );
		int eEnd = chunk_scan( isEnd, smem, &tEnd );
		if ( k < nOps )
		{
			int2 s = w.cshape[c];
			if ( isBegin )
			{
				int e = runBegin + eBegin;
				if ( e < w.eventCap )
				{
					w.beginEv[2 * e] = s.x;
					w.beginEv[2 * e + 1] = s.y;
				}
			}
			if ( isEnd )
			{
				int e = runEnd + eEnd;
				if ( e < w.eventCap )
				{
					w.endEv[2 * e] = s.x;
					w.endEv[2 * e + 1] = s.y;
				}
			}
			if ( kind == 0 )
			{
				w.contactFree[F + runFree + eFree] = c;
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
		runFree += tFree;
		runBegin += tBegin;
		runEnd += tEnd;
		__syncthreads();
	}
	if ( threadIdx.x == 0 )
	{
		w.sc->contactFreeCount = F + runFree;
		w.sc->beginCount = min( runBegin, w.eventCap );
		w.sc->endCount = min( runEnd, w.eventCap );
		if ( runBegin > w.eventCap || runEnd > w.eventCap )
			atomicOr( &w.sc->error, ERR_EVENT_CAPACITY );
		w.sc->opCount = 0;
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
		if ( color == F2D_OVERFLOW )
		{
			w.overflowJoints[w.sc->overflowJointCount] = j;
			w.sc->overflowJointCount += 1;
		}
	}
}

void launch_graph( DWorld& w, StepScratch& s, cudaStream_t st )
{
	k_color_ops<<<1, GRAPH_THREADS, 0, st>>>( w, s.tmpA );
}

void launch_joint_ops( DWorld& w, cudaStream_t st )
{
	if ( w.pendingJointCount > 0 )
		k_joint_ops<<<1, 1, 0, st>>>( w, w.pendingJointCount );
}
