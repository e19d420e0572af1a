// Shared launch helpers and the per-phase launch entry points of the step.
#pragma once

#include "dworld.cuh"

#include <cuda_runtime.h>

#define F2D_SMS 152 // GB300: 2 dies x 76 SMs

// Grid for a grid-stride kernel over `cap` items: whole waves of the
// 152 SMs, at most 8 resident 256-thread blocks per SM.
static inline int grid_for( int cap )
{
	int blocks = ( cap + 255 ) / 256;
	if ( blocks < 1 )
		blocks = 1;
	int maxBlocks = F2D_SMS * 8;
	if ( blocks > maxBlocks )
		blocks = maxBlocks;
	return blocks;
}

// Step scratch owned by the host world; device pointers only.
struct StepScratch
{
	int* tmpA;	  // >= max(shapeCap, contactCap, bodyCap) ints
	int* tmpB;
	int* scanTmp; // scan tile sums
	unsigned long long* scanState; // look-back scan tile states
	int sortBlocks32, sortBlocks64; // co-resident grids of the one-launch sorts
	float4* bounds;
	int boundsBlocks;
	int shapeIdBits;
	int solverBlocks;  // persistent solver grid (co-resident)
	int solverThreads;
	int clusterCapacity; // bodies the cluster solver takes (0: cooperative solver only)
	int solverBlocks256; // grid of the 256-thread variant of the grid-wide solver
	int solverVariant;	 // SOLVER_* (the autotuner's choice; results never depend on it)
	int ptBlocks;		 // co-resident grid of the tree rebuild's cooperative levels
	cudaEvent_t evSolveStart; // recorded right before the cooperative solver launch when non-null
	// streams beside the world's own for independent launches of one phase
	// (the manifold classes), with their fork and join events
	cudaStream_t side[4];
	cudaEvent_t sideFork, sideJoin[4];
	// the tree rebuild's stream, its fork and join, and (profiling only,
	// else null) the events around it
	cudaStream_t rebuild;
	cudaEvent_t rebuildFork, rebuildJoin, rebuildT0, rebuildT1;
};

// solver variants: same arithmetic, different launch shapes
#define SOLVER_AUTO 0	 // cluster solver up to 2e4 bodies, else grid-wide with 512-thread blocks
#define SOLVER_CLUSTER 1 // one thread-block cluster (when the bodies fit its shared memory)
#define SOLVER_GRID512 2 // grid-wide, one 512-thread block per SM
#define SOLVER_GRID256 3 // grid-wide, two 256-thread blocks per SM

// A host hook runs between launches when the world has user callbacks
// (the stream is synchronised by the hook itself).
typedef void ( *HostHook )( void* context );
void launch_broadphase( DWorld& w, StepScratch& s, cudaStream_t st, int planMode, HostHook pairHook = nullptr,
						void* hookContext = nullptr );
void launch_narrowphase( DWorld& w, StepScratch& s, cudaStream_t st, HostHook preSolveHook = nullptr,
						 void* hookContext = nullptr );
void launch_graph( DWorld& w, StepScratch& s, cudaStream_t st );
void launch_solver( DWorld& w, StepScratch& s, cudaStream_t st, float dt, int subSteps );
void launch_finalize( DWorld& w, StepScratch& s, cudaStream_t st, float dt, HostHook ccdHook = nullptr,
					  void* hookContext = nullptr );
void launch_sensors( DWorld& w, StepScratch& s, cudaStream_t st );
void launch_joint_ops( DWorld& w, cudaStream_t st );
int solver_max_blocks( int threads );
// islands and sleeping (island.cu; worlds with sleeping enabled)
void launch_isl_create( DWorld& w, cudaStream_t st );
void launch_isl_new_contacts( DWorld& w, StepScratch& s, cudaStream_t st, int planMode );
void launch_isl_ops( DWorld& w, StepScratch& s, cudaStream_t st, const int* gkind );
void launch_isl_split( DWorld& w, cudaStream_t st );
void launch_isl_sleep( DWorld& w, cudaStream_t st, unsigned long long* scanState );
void launch_isl_api( DWorld& w, cudaStream_t st, int op, int body );
// destroy path (island.cu), serial launches between steps: the contacts of a
// body in its contact-list order (only those of `shape` / with body `other`
// when >= 0; `list` holds contactCap ints), one joint, a body's island and
// solver-set records, one proxy out of the move array
void launch_destroy_contacts_of( DWorld& w, cudaStream_t st, int body, int shape, int other, int wake, int* list );
void launch_destroy_joint( DWorld& w, cudaStream_t st, int joint, int wake );
void launch_destroy_body_records( DWorld& w, cudaStream_t st, int body );
// type changes, disable and enable (island.cu), serial launches between steps
void launch_body_set_type( DWorld& w, cudaStream_t st, int body, int type );
void launch_body_disable( DWorld& w, cudaStream_t st, int body );
void launch_body_enable( DWorld& w, cudaStream_t st, int body );
void launch_unbuffer_move( DWorld& w, cudaStream_t st, int shape );
// microseconds per grid barrier on the grid-wide solver's grid (n barriers timed)
float solver_barrier_probe( StepScratch& s, cudaStream_t st, unsigned* counter, int* err, int n );
// b2Shape_TestPoint on the device row of one shape; *out (device) = 0 or 1
void launch_shape_test_point( DWorld& w, cudaStream_t st, int shape, float x, float y, int* out );
void launch_isl_wake_marked( DWorld& w, cudaStream_t st, const int* shapeMarks, int shapeCount );
void launch_explode( DWorld& w, cudaStream_t st, int* hit, unsigned long long mask, float x, float y, float radius,
					 float falloff, float impulsePerLength );
void launch_isl_fix_flags( DWorld& w, cudaStream_t st, int n );
void launch_learned_warm_start( DWorld& w, cudaStream_t st );
void launch_record_samples( DWorld& w, cudaStream_t st );
int solver_cluster_capacity();
// the reference's broadphase trees and the move array (proxytree.cu)
int pt_large_blocks();
void launch_pt_host_moves( DWorld& w, StepScratch& s, cudaStream_t st );
void launch_pt_decode( DWorld& w, cudaStream_t st );
void launch_pt_rebuild( DWorld& w, StepScratch& s, cudaStream_t st );
void launch_pt_moves( DWorld& w, StepScratch& s, cudaStream_t st );
void launch_pt_ranks( DWorld& w, cudaStream_t st, int t );
