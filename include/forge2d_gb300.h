/*
 * forge2d_gb300 -- C ABI of the GPU world step.
 *
 * A drop-in for the part of forge2d's backend seam that drives the Box2D v3
 * world step: `abstract interface class RawBox2D`
 * (packages/forge2d/lib/src/backend/raw_box2d.dart:10). Each entry point
 * below names the RawBox2D method it replaces and the native Box2D call that
 * method makes today through dart:ffi (raw_box2d_ffi.dart). The seam's rules
 * hold (packages/forge2d/lib/src/backend/README.md:21-39): primitives only,
 * ids packed into 32-bit ints -- world id = index1 | generation << 16; body,
 * shape and joint ids are (index1, worldAndGeneration = world0 |
 * generation << 16) pairs -- no callbacks, definition structs flattened,
 * results written into caller-provided buffers.
 *
 * Errors: functions never trap. Invalid ids are ignored (getters return 0),
 * creation returns 0 and leaves the id outputs at 0, f2d_world_step returns
 * a nonzero F2D_STATUS_* bit set when a device capacity or wait limit was
 * hit (the step's results are then incomplete and the world should be
 * recreated with larger capacities).
 *
 * Threading: a world belongs to one host thread; every call is synchronous
 * with respect to the caller except f2d_world_step, which enqueues the step
 * on the world's CUDA stream (getters and event readers synchronise).
 */
#ifndef FORGE2D_GB300_H
#define FORGE2D_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined( _WIN32 )
#define F2D_API __declspec( dllexport )
#else
#define F2D_API __attribute__( ( visibility( "default" ) ) )
#endif

/* Mirrors RawBox2D.createWorld's named parameters (raw_box2d.dart:18-29). */
typedef struct f2d_world_def
{
	double gravityX, gravityY;
	double restitutionThreshold;
	double hitEventThreshold;
	double contactHertz;
	double contactDampingRatio;
	double maxContactPushSpeed;
	double maximumLinearSpeed;
	int32_t enableSleep;
	int32_t enableContinuous;
} f2d_world_def;

/* Mirrors RawBox2D.createBody's named parameters (raw_box2d.dart:71-91);
 * type is the BodyType index (0 static, 1 kinematic, 2 dynamic). */
typedef struct f2d_body_def
{
	int32_t type;
	int32_t pad0;
	double positionX, positionY;
	double rotationCos, rotationSin;
	double linearVelocityX, linearVelocityY;
	double angularVelocity;
	double linearDamping;
	double angularDamping;
	double gravityScale;
	double sleepThreshold;
	int32_t enableSleep;
	int32_t isAwake;
	int32_t fixedRotation;
	int32_t isBullet;
	int32_t isEnabled;
	int32_t allowFastRotation;
} f2d_body_def;

/* Mirrors RawShapeDef (raw_box2d_ffi.dart:564-584 maps it to b2ShapeDef).
 * 64-bit filter masks follow the seam's sign-extension rule: -1 = all bits. */
typedef struct f2d_shape_def
{
	double friction;
	double restitution;
	double rollingResistance;
	double tangentSpeed;
	double density;
	int64_t categoryBits;
	int64_t maskBits;
	int32_t groupIndex;
	int32_t userMaterialId;
	int32_t isSensor;
	int32_t enableSensorEvents;
	int32_t enableContactEvents;
	int32_t enableHitEvents;
	int32_t enablePreSolveEvents;
	int32_t invokeContactCreation;
	int32_t updateBodyMass;
	int32_t pad0;
} f2d_shape_def;

/* Mirrors World.createRevoluteJoint / RawBox2D.createRevoluteJoint
 * (packages/forge2d/lib/src/api/world.dart:297-321). */
typedef struct f2d_revolute_def
{
	int32_t bodyAIndex1, bodyAWorldAndGeneration;
	int32_t bodyBIndex1, bodyBWorldAndGeneration;
	double localAnchorAX, localAnchorAY;
	double localAnchorBX, localAnchorBY;
	double referenceAngle;
	double targetAngle;
	int32_t enableSpring;
	int32_t pad0;
	double hertz;
	double dampingRatio;
	int32_t enableLimit;
	int32_t pad1;
	double lowerAngle, upperAngle;
	int32_t enableMotor;
	int32_t pad2;
	double maxMotorTorque;
	double motorSpeed;
	double drawSize;
	int32_t collideConnected;
	int32_t pad3;
} f2d_revolute_def;

/* Mirrors RawBox2D.create{Distance,Filter,Motor,Mouse,Prismatic,Weld,Wheel}
 * Joint (raw_box2d.dart:582-712 -> b2Create*Joint, joint.c:400-720): one
 * definition for every type; fields the type does not use are ignored. The
 * bodies are (index1, worldAndGeneration) id pairs. */
#define F2D_JOINT_WELD 2
#define F2D_JOINT_DISTANCE 3
#define F2D_JOINT_PRISMATIC 4
#define F2D_JOINT_WHEEL 5
#define F2D_JOINT_MOTOR 6
#define F2D_JOINT_MOUSE 7
#define F2D_JOINT_FILTER 8
typedef struct f2d_joint_def
{
	int32_t type;
	int32_t bodyAIndex1, bodyAWorldAndGeneration;
	int32_t bodyBIndex1, bodyBWorldAndGeneration;
	int32_t collideConnected;
	double localAnchorAX, localAnchorAY;
	double localAnchorBX, localAnchorBY;
	double referenceAngle;
	/* weld */
	double linearHertz, linearDampingRatio;
	double angularHertz, angularDampingRatio;
	/* distance */
	double length, minLength, maxLength;
	double hertz, dampingRatio;
	double maxMotorForce, motorSpeed;
	int32_t enableSpring, enableLimit, enableMotor, pad0;
	/* prismatic and wheel */
	double localAxisAX, localAxisAY;
	double targetTranslation, lowerTranslation, upperTranslation;
	double maxMotorTorque;
	/* motor (maxForce also the mouse joint's) */
	double linearOffsetX, linearOffsetY, angularOffset;
	double maxForce, maxTorque, correctionFactor;
	/* mouse */
	double targetX, targetY;
} f2d_joint_def;

#define F2D_STATUS_OK 0
#define F2D_STATUS_CONTACT_CAPACITY 0x1
#define F2D_STATUS_PAIR_CAPACITY 0x2
#define F2D_STATUS_BARRIER_TIMEOUT 0x4
#define F2D_STATUS_PLAN_MISMATCH 0x8
#define F2D_STATUS_OP_CAPACITY 0x10
#define F2D_STATUS_COLOR_ROUNDS 0x20
#define F2D_STATUS_EVENT_CAPACITY 0x40
#define F2D_STATUS_TREE 0x80
#define F2D_STATUS_INVALID 0x100
#define F2D_STATUS_CUDA 0x200

/* ---- world lifecycle ---------------------------------------------------- */

/* RawBox2D.createWorld (raw_box2d.dart:18; raw_box2d_ffi.dart:67 -> b2CreateWorld).
 * Returns the packed world id, 0 on failure (no CUDA device, table full). */
F2D_API int32_t f2d_create_world( const f2d_world_def* def );
/* RawBox2D.destroyWorld (raw_box2d.dart:32 -> b2DestroyWorld). */
F2D_API void f2d_destroy_world( int32_t worldId );
/* RawBox2D.worldIsValid (raw_box2d.dart:35 -> b2World_IsValid). */
F2D_API int32_t f2d_world_is_valid( int32_t worldId );
/* RawBox2D.worldStep (raw_box2d.dart:39; raw_box2d_ffi.dart:103 -> b2World_Step).
 * Returns F2D_STATUS_* bits of the previous device step (checked lazily so
 * that consecutive steps do not synchronise). */
F2D_API int32_t f2d_world_step( int32_t worldId, double timeStep, int32_t subStepCount );
/* Blocks until the world's enqueued work is done; returns the status bits. */
F2D_API int32_t f2d_world_sync( int32_t worldId );
/* RawBox2D.worldSetGravity / worldGetGravity (raw_box2d.dart:42-45). */
F2D_API void f2d_world_set_gravity( int32_t worldId, double x, double y );
F2D_API void f2d_world_get_gravity( int32_t worldId, double* x, double* y );
/* RawBox2D.worldEnableSleeping / worldIsSleepingEnabled (raw_box2d.dart:49-52). */
F2D_API void f2d_world_enable_sleeping( int32_t worldId, int32_t enabled );
F2D_API int32_t f2d_world_is_sleeping_enabled( int32_t worldId );
/* RawBox2D.worldEnableContinuous / worldIsContinuousEnabled (raw_box2d.dart:55-58). */
F2D_API void f2d_world_enable_continuous( int32_t worldId, int32_t enabled );
F2D_API int32_t f2d_world_is_continuous_enabled( int32_t worldId );

/* ---- batched form (no reference counterpart) ---------------------------
 * Thousands of independent worlds advance together as sub-worlds of one
 * world: every step phase, including the persistent solver kernel, runs once
 * for all of them. Bodies created after f2d_world_begin_subworld belong to
 * the new sub-world and feel its gravity; shapes of different sub-worlds
 * never make contacts. Returns the sub-world index, -1 for an invalid world. */
F2D_API int32_t f2d_world_begin_subworld( int32_t worldId, double gravityX, double gravityY );
F2D_API int32_t f2d_world_subworld_count( int32_t worldId );

/* ---- bodies ------------------------------------------------------------- */

/* RawBox2D.createBody (raw_box2d.dart:71; raw_box2d_ffi.dart:135 -> b2CreateBody). */
F2D_API int32_t f2d_create_body( int32_t worldId, const f2d_body_def* def, int32_t* index1,
								 int32_t* worldAndGeneration );
/* RawBox2D.destroyBody (raw_box2d.dart:96 -> b2DestroyBody, body.c:343):
 * its joints (waking their bodies), its contacts (waking touching pairs),
 * its shapes with their sensors and proxies, its chains, its island and
 * solver-set records; ids go back to LIFO pools and keep their generation.
 * End events of destroyed touching contacts (and of destroyed sensors'
 * visitors) are reported with the next step's, ahead of its own. */
F2D_API void f2d_destroy_body( int32_t index1, int32_t worldAndGeneration );
/* RawBox2D.bodyIsValid (raw_box2d.dart:99 -> b2Body_IsValid). */
F2D_API int32_t f2d_body_is_valid( int32_t index1, int32_t worldAndGeneration );
/* RawBox2D.bodyGetPosition / bodyGetRotation (raw_box2d.dart:102-106). */
F2D_API void f2d_body_get_position( int32_t index1, int32_t worldAndGeneration, double* x, double* y );
F2D_API void f2d_body_get_rotation( int32_t index1, int32_t worldAndGeneration, double* c, double* s );
/* RawBox2D.bodySetTransform (raw_box2d.dart:109 -> b2Body_SetTransform). */
F2D_API void f2d_body_set_transform( int32_t index1, int32_t worldAndGeneration, double px, double py, double c,
									 double s );
/* RawBox2D.bodyGet/SetLinearVelocity, bodyGet/SetAngularVelocity (raw_box2d.dart:119-133). */
F2D_API void f2d_body_get_linear_velocity( int32_t index1, int32_t worldAndGeneration, double* x, double* y );
F2D_API void f2d_body_set_linear_velocity( int32_t index1, int32_t worldAndGeneration, double x, double y );
F2D_API double f2d_body_get_angular_velocity( int32_t index1, int32_t worldAndGeneration );
F2D_API void f2d_body_set_angular_velocity( int32_t index1, int32_t worldAndGeneration, double w );
/* RawBox2D.bodyApplyForce / bodyApplyForceToCenter / bodyApplyTorque /
 * bodyApplyLinearImpulse / bodyApplyLinearImpulseToCenter /
 * bodyApplyAngularImpulse (raw_box2d.dart:136-190). wake = 1 wakes a
 * sleeping body first; the push is dropped on a body that stays asleep, as
 * in body.c:1000-1110. */
F2D_API void f2d_body_apply_force( int32_t index1, int32_t worldAndGeneration, double fx, double fy, double px,
								   double py, int32_t wake );
F2D_API void f2d_body_apply_force_to_center( int32_t index1, int32_t worldAndGeneration, double fx, double fy,
											 int32_t wake );
F2D_API void f2d_body_apply_torque( int32_t index1, int32_t worldAndGeneration, double torque, int32_t wake );
F2D_API void f2d_body_apply_linear_impulse( int32_t index1, int32_t worldAndGeneration, double ix, double iy,
											double px, double py, int32_t wake );
F2D_API void f2d_body_apply_linear_impulse_to_center( int32_t index1, int32_t worldAndGeneration, double ix,
													  double iy, int32_t wake );
F2D_API void f2d_body_apply_angular_impulse( int32_t index1, int32_t worldAndGeneration, double impulse,
											 int32_t wake );
/* RawBox2D.bodyGetMass / bodyGetRotationalInertia / bodyGetType (raw_box2d.dart:192-217). */
F2D_API double f2d_body_get_mass( int32_t index1, int32_t worldAndGeneration );
F2D_API double f2d_body_get_rotational_inertia( int32_t index1, int32_t worldAndGeneration );
F2D_API int32_t f2d_body_get_type( int32_t index1, int32_t worldAndGeneration );
F2D_API int32_t f2d_body_is_awake( int32_t index1, int32_t worldAndGeneration );
/* RawBox2D.bodySetAwake (raw_box2d.dart:232 -> b2Body_SetAwake): wakes the
 * body's sleeping set, or puts its island to sleep (splitting it first when
 * constraints were removed). Worlds created with sleeping off keep every body
 * awake and ignore it. */
F2D_API void f2d_body_set_awake( int32_t index1, int32_t worldAndGeneration, int32_t awake );
/* RawBox2D.bodySetType (raw_box2d.dart:220 -> b2Body_SetType, body.c:1036):
 * type 0 static, 1 kinematic, 2 dynamic. The body's contacts end without
 * waking anything, its joints move between the static and awake sets (and
 * re-take graph colours), its proxies move to the new type's tree (forced
 * pair search) and its mass data is recomputed. A disabled body only changes
 * type and mass. One deviation: a removal from the constraint graph clears
 * only the colour bits the joint's colouring set, so when a static body
 * holding two or more joints of the graph turns non-static its joints take
 * distinct colours where the reference can give two of them one colour. */
F2D_API void f2d_body_set_type( int32_t index1, int32_t worldAndGeneration, int32_t type );
/* RawBox2D.bodyDisable / bodyEnable (raw_box2d.dart:254-257 -> b2Body_Disable
 * / b2Body_Enable, body.c:1557-1700): disabling ends the body's contacts
 * (waking the bodies they touched), removes its proxies and moves it and its
 * joints to the disabled set; enabling puts it back in the static or awake
 * set with new proxies (forced pair search) and re-links its joints whose
 * other body is enabled. */
F2D_API void f2d_body_disable( int32_t index1, int32_t worldAndGeneration );
F2D_API void f2d_body_enable( int32_t index1, int32_t worldAndGeneration );
/* RawBox2D.bodyIsSleepEnabled / bodyEnableSleep (raw_box2d.dart:235-242 ->
 * b2Body_IsSleepEnabled / b2Body_EnableSleep; disabling wakes the body). */
F2D_API int32_t f2d_body_is_sleep_enabled( int32_t index1, int32_t worldAndGeneration );
F2D_API void f2d_body_enable_sleep( int32_t index1, int32_t worldAndGeneration, int32_t enabled );
/* RawBox2D.bodyGetSleepThreshold / bodySetSleepThreshold (raw_box2d.dart:245-248). */
F2D_API double f2d_body_get_sleep_threshold( int32_t index1, int32_t worldAndGeneration );
F2D_API void f2d_body_set_sleep_threshold( int32_t index1, int32_t worldAndGeneration, double value );

/* ---- shapes ------------------------------------------------------------- */

/* RawBox2D.createCircleShape (raw_box2d.dart:327; raw_box2d_ffi.dart:588 -> b2CreateCircleShape). */
F2D_API int32_t f2d_create_circle_shape( int32_t bodyIndex1, int32_t bodyWorldAndGeneration, const f2d_shape_def* def,
										 double centerX, double centerY, double radius, int32_t* index1,
										 int32_t* worldAndGeneration );
/* RawBox2D.createCapsuleShape (raw_box2d.dart:336; raw_box2d_ffi.dart:612 -> b2CreateCapsuleShape). */
F2D_API int32_t f2d_create_capsule_shape( int32_t bodyIndex1, int32_t bodyWorldAndGeneration,
										  const f2d_shape_def* def, double center1X, double center1Y,
										  double center2X, double center2Y, double radius, int32_t* index1,
										  int32_t* worldAndGeneration );
/* RawBox2D.createSegmentShape (raw_box2d.dart:348; raw_box2d_ffi.dart:640 -> b2CreateSegmentShape). */
F2D_API int32_t f2d_create_segment_shape( int32_t bodyIndex1, int32_t bodyWorldAndGeneration,
										  const f2d_shape_def* def, double point1X, double point1Y,
										  double point2X, double point2Y, int32_t* index1,
										  int32_t* worldAndGeneration );
/* RawBox2D.createBoxShape (raw_box2d.dart:363; raw_box2d_ffi.dart:666 ->
 * b2MakeOffsetRoundedBox + b2CreatePolygonShape). */
F2D_API int32_t f2d_create_box_shape( int32_t bodyIndex1, int32_t bodyWorldAndGeneration, const f2d_shape_def* def,
									  double halfWidth, double halfHeight, double centerX, double centerY,
									  double rotationCos, double rotationSin, double radius, int32_t* index1,
									  int32_t* worldAndGeneration );
/* RawBox2D.createPolygonShape (raw_box2d.dart:380; raw_box2d_ffi.dart:696 ->
 * b2ComputeHull + b2MakePolygon + b2CreatePolygonShape). points packed
 * x0,y0,x1,y1,...; returns 0 for a degenerate hull (forge2d throws
 * ArgumentError there, raw_box2d_ffi.dart:717-721). */
F2D_API int32_t f2d_create_polygon_shape( int32_t bodyIndex1, int32_t bodyWorldAndGeneration,
										  const f2d_shape_def* def, const double* points, int32_t count,
										  double radius, int32_t* index1, int32_t* worldAndGeneration );
/* RawBox2D.createChain (raw_box2d.dart:537 -> b2CreateChain, shape.c:339):
 * points packed [x0, y0, x1, y1, ...], count >= 4; materials six values each
 * (friction, restitution, rollingResistance, tangentSpeed, userMaterialId,
 * customColor), one or one per point. Returns the chain id pair. */
F2D_API int32_t f2d_create_chain( int32_t bodyIndex1, int32_t bodyWorldAndGeneration, const double* points,
								  int32_t count, const double* materials, int32_t materialCount, int64_t categoryBits,
								  int64_t maskBits, int32_t groupIndex, int32_t isLoop, int32_t enableSensorEvents,
								  int32_t* index1, int32_t* worldAndGeneration );
/* RawBox2D.chainGetSegments (raw_box2d.dart:571): the segment shape id pairs
 * (index1, worldAndGeneration) in creation order; returns the count. */
F2D_API int32_t f2d_chain_get_segments( int32_t index1, int32_t worldAndGeneration, int32_t* out2,
										int32_t capacity );
/* RawBox2D.destroyShape (raw_box2d.dart:390 -> b2DestroyShape, shape.c:318):
 * proxy, contacts (waking), sensor; the body's mass is recomputed when
 * updateBodyMass is non-zero. */
F2D_API void f2d_destroy_shape( int32_t index1, int32_t worldAndGeneration, int32_t updateBodyMass );
/* RawBox2D.destroyChain (raw_box2d.dart:550 -> b2DestroyChain, shape.c:488):
 * every segment shape in creation order, then the chain id. */
F2D_API void f2d_destroy_chain( int32_t index1, int32_t worldAndGeneration );
/* RawBox2D.shapeIsValid / shapeGetType (raw_box2d.dart:397-400). */
F2D_API int32_t f2d_shape_is_valid( int32_t index1, int32_t worldAndGeneration );
F2D_API int32_t f2d_shape_get_type( int32_t index1, int32_t worldAndGeneration );

/* ---- joints ------------------------------------------------------------- */

/* RawBox2D.createRevoluteJoint (world.dart:297-321 -> b2CreateRevoluteJoint, joint.c:507). */
/* RawBox2D.create{Distance,Filter,Motor,Mouse,Prismatic,Weld,Wheel}Joint
 * (raw_box2d.dart:582-712). */
F2D_API int32_t f2d_create_joint( int32_t worldId, const f2d_joint_def* def, int32_t* index1,
								  int32_t* worldAndGeneration );
/* RawBox2D.mouseJointSetTarget (raw_box2d.dart:913 -> b2MouseJoint_SetTarget,
 * mouse_joint.c:14): takes effect at the next step; wakes nothing. */
F2D_API void f2d_mouse_joint_set_target( int32_t index1, int32_t worldAndGeneration, double x, double y );
/* RawBox2D.{revolute,prismatic,wheel,distance}JointEnableMotor / SetMotorSpeed /
 * SetMaxMotorTorque|Force (raw_box2d.dart:823-850 and the revolute, prismatic
 * and wheel sections): the motor's state, speed and maximum torque (revolute,
 * wheel) or force (prismatic, distance) in one call; takes effect at the next
 * step; wakes nothing. */
F2D_API void f2d_joint_set_motor( int32_t index1, int32_t worldAndGeneration, int32_t enable, double speed,
								  double maxMotor );
/* RawBox2D.jointGetConstraintForce / jointGetConstraintTorque (raw_box2d.dart:
 * 748-751 -> b2Joint_GetConstraintForce / Torque, joint.c:1061): the last
 * step's constraint force and torque; out3 = force.x, force.y, torque. */
F2D_API void f2d_joint_get_constraint( int32_t index1, int32_t worldAndGeneration, float* out3 );
/* RawBox2D.{revolute,prismatic,wheel}JointEnableLimit / SetLimits: the limit's
 * state and bounds (angles for the revolute joint, translations otherwise)
 * in one call; takes effect at the next step; wakes nothing. */
F2D_API void f2d_joint_set_limits( int32_t index1, int32_t worldAndGeneration, int32_t enable, double lower,
								   double upper );
F2D_API int32_t f2d_create_revolute_joint( int32_t worldId, const f2d_revolute_def* def, int32_t* index1,
										   int32_t* worldAndGeneration );
F2D_API int32_t f2d_joint_is_valid( int32_t index1, int32_t worldAndGeneration );
/* RawBox2D.destroyJoint (raw_box2d.dart:714 -> b2DestroyJoint, joint.c:808):
 * out of the graph, island and solver set; wakes its bodies. A joint created
 * with collideConnected false (all types but mouse and filter) destroys the
 * contacts between its bodies, without waking (joint.c:313-351). */
F2D_API void f2d_destroy_joint( int32_t index1, int32_t worldAndGeneration );
/* RawBox2D.jointSetCollideConnected / jointGetCollideConnected
 * (raw_box2d.dart:738 / :735 -> b2Joint_SetCollideConnected, joint.c:980-1022): allowing collision
 * buffers the proxies of the body with fewer shapes for the next pair
 * search; forbidding it destroys the contacts between the bodies. */
F2D_API void f2d_joint_set_collide_connected( int32_t index1, int32_t worldAndGeneration, int32_t flag );
F2D_API int32_t f2d_joint_get_collide_connected( int32_t index1, int32_t worldAndGeneration );

/* ---- properties ---------------------------------------------------------
 * The RawBox2D getters and setters without a call of their own go through
 * one get and one set per kind, the property chosen by a code named for the
 * RawBox2D method pair (raw_box2d.dart line beside each). Gets return 0 for
 * an invalid id or a code the object does not have; sets ignore them, and
 * ignore values the reference's setter asserts against (negative damping,
 * NaN, ...). Pairs (limits, length range, linear offset) are set with both
 * values at once: value = first, value2 = second. */

/* bodies: f2d_body_get_param / f2d_body_set_param */
#define F2D_BODY_LINEAR_DAMPING 1	/* bodyGet/SetLinearDamping :282-291 */
#define F2D_BODY_ANGULAR_DAMPING 2	/* bodyGet/SetAngularDamping :288-291 */
#define F2D_BODY_GRAVITY_SCALE 3	/* bodyGet/SetGravityScale :276-279 */
#define F2D_BODY_BULLET 4			/* bodyIsBullet / bodySetBullet :270-273 */
#define F2D_BODY_FIXED_ROTATION 5	/* bodyIsFixedRotation / bodySetFixedRotation :260-263 */
#define F2D_BODY_ENABLED 6			/* bodyIsEnabled / bodyEnable / bodyDisable :251-257 */
#define F2D_BODY_TYPE 7				/* bodyGetType / bodySetType :217-220 */
#define F2D_BODY_LOCAL_CENTER_X 8	/* bodyGetLocalCenterOfMass :198 */
#define F2D_BODY_LOCAL_CENTER_Y 9
#define F2D_BODY_WORLD_CENTER_X 10	/* bodyGetWorldCenterOfMass :201 */
#define F2D_BODY_WORLD_CENTER_Y 11
F2D_API double f2d_body_get_param( int32_t index1, int32_t worldAndGeneration, int32_t code );
F2D_API void f2d_body_set_param( int32_t index1, int32_t worldAndGeneration, int32_t code, double value );
/* RawBox2D.bodyGetWorldPoint / bodyGetLocalPoint (raw_box2d.dart:298-311). */
F2D_API void f2d_body_get_world_point( int32_t index1, int32_t worldAndGeneration, double x, double y, double* ox,
									   double* oy );
F2D_API void f2d_body_get_local_point( int32_t index1, int32_t worldAndGeneration, double x, double y, double* ox,
									   double* oy );
/* RawBox2D.bodySetMassData / bodyApplyMassFromShapes (raw_box2d.dart:204-214
 * -> b2Body_SetMassData, body.c:917; b2Body_ApplyMassFromShapes). */
F2D_API void f2d_body_set_mass_data( int32_t index1, int32_t worldAndGeneration, double mass,
									 double rotationalInertia, double centerX, double centerY );
F2D_API void f2d_body_apply_mass_from_shapes( int32_t index1, int32_t worldAndGeneration );
/* RawBox2D.bodyGetName / bodySetName (raw_box2d.dart:223-226): up to 31
 * bytes kept (b2Body_SetName, body.c:1160); null or "" clears it. get copies
 * the name, zero-terminated, into out (capacity bytes) and returns its
 * length. */
F2D_API void f2d_body_set_name( int32_t index1, int32_t worldAndGeneration, const char* name );
F2D_API int32_t f2d_body_get_name( int32_t index1, int32_t worldAndGeneration, char* out, int32_t capacity );
/* RawBox2D.bodyGetShapes / bodyGetJoints (raw_box2d.dart:315-319): id pairs
 * in the body's list order (newest first); returns the count. */
F2D_API int32_t f2d_body_get_shapes( int32_t index1, int32_t worldAndGeneration, int32_t* out2, int32_t capacity );
F2D_API int32_t f2d_body_get_joints( int32_t index1, int32_t worldAndGeneration, int32_t* out2, int32_t capacity );

/* shapes: f2d_shape_get_param / f2d_shape_set_param (flag = updateBodyMass
 * for the density) */
#define F2D_SHAPE_DENSITY 1			/* shapeGetDensity / shapeSetDensity :409-417 */
#define F2D_SHAPE_FRICTION 2		/* shapeGet/SetFriction :420-423 */
#define F2D_SHAPE_RESTITUTION 3		/* shapeGet/SetRestitution :426-433 */
#define F2D_SHAPE_SENSOR 4			/* shapeIsSensor :406 (get) */
#define F2D_SHAPE_SENSOR_EVENTS 5	/* shapeAreSensorEventsEnabled / shapeEnableSensorEvents :448-455 */
#define F2D_SHAPE_CONTACT_EVENTS 6	/* :458-465 */
#define F2D_SHAPE_HIT_EVENTS 7		/* :468-475 */
#define F2D_SHAPE_PRESOLVE_EVENTS 8 /* :478-485 */
#define F2D_SHAPE_CATEGORY 9		/* shapeGetFilter :436 (get) */
#define F2D_SHAPE_MASK 10
#define F2D_SHAPE_GROUP 11
F2D_API double f2d_shape_get_param( int32_t index1, int32_t worldAndGeneration, int32_t code );
F2D_API void f2d_shape_set_param( int32_t index1, int32_t worldAndGeneration, int32_t code, double value,
								  int32_t flag );
/* RawBox2D.shapeGetBody (raw_box2d.dart:403). */
F2D_API int32_t f2d_shape_get_body( int32_t index1, int32_t worldAndGeneration, int32_t* bodyIndex1,
									int32_t* bodyWorldAndGeneration );
/* RawBox2D.shapeSetFilter (raw_box2d.dart:439 -> b2Shape_SetFilter,
 * shape.c:1197): a change of category or mask re-creates the proxy (its
 * contacts end, the bodies wake); a group change alone keeps it. */
F2D_API void f2d_shape_set_filter( int32_t index1, int32_t worldAndGeneration, int64_t categoryBits, int64_t maskBits,
								   int32_t groupIndex );
/* RawBox2D.shapeTestPoint (raw_box2d.dart:488 -> b2Shape_TestPoint). */
F2D_API int32_t f2d_shape_test_point( int32_t index1, int32_t worldAndGeneration, double x, double y );
/* RawBox2D.shapeGetCircle / GetCapsule / GetSegment / GetChainSegment /
 * GetPolygon (raw_box2d.dart:491-520): the shape's local geometry; returns
 * the number of floats written to out (circle 3: center, radius; capsule 5:
 * center1, center2, radius; segment and chain segment 4: point1, point2;
 * polygon 2 * count + 1: vertices, then the radius), 0 for another type. */
F2D_API int32_t f2d_shape_get_geometry( int32_t index1, int32_t worldAndGeneration, int32_t type, double* out,
										int32_t capacity );
/* RawBox2D.shapeGetAabb (raw_box2d.dart:524 -> b2Shape_GetAABB): the
 * shape's current box (lower.xy, upper.xy). */
F2D_API void f2d_shape_get_aabb( int32_t index1, int32_t worldAndGeneration, double* out4 );

/* chains: RawBox2D.chainIsValid / chainSet/GetFriction / Restitution
 * (raw_box2d.dart:553-569); the set reaches every segment (shape.c:1476). */
F2D_API int32_t f2d_chain_is_valid( int32_t index1, int32_t worldAndGeneration );
F2D_API double f2d_chain_get_param( int32_t index1, int32_t worldAndGeneration, int32_t code );
F2D_API void f2d_chain_set_param( int32_t index1, int32_t worldAndGeneration, int32_t code, double value );

/* joints: f2d_joint_get_param / f2d_joint_set_param. The codes that belong
 * to each type follow the type's RawBox2D methods; setters clear the
 * impulses the reference's setters clear and wake nothing. */
#define F2D_JP_TYPE 1				/* jointGetType :720 (b2JointType values) */
#define F2D_JP_LOCAL_ANCHOR_AX 2	/* jointGetLocalAnchorA / B :729-732 */
#define F2D_JP_LOCAL_ANCHOR_AY 3
#define F2D_JP_LOCAL_ANCHOR_BX 4
#define F2D_JP_LOCAL_ANCHOR_BY 5
#define F2D_JP_SPRING_ENABLED 6		/* {distance,prismatic,revolute,wheel}JointIsSpringEnabled / EnableSpring */
#define F2D_JP_SPRING_HERTZ 7		/* ...Get/SetSpringHertz (and mouse) */
#define F2D_JP_SPRING_DAMPING 8		/* ...Get/SetSpringDampingRatio (and mouse) */
#define F2D_JP_TARGET 9				/* revoluteJointGet/SetTargetAngle, prismaticJointGet/SetTargetTranslation */
#define F2D_JP_LIMIT_ENABLED 10		/* {distance,prismatic,revolute,wheel}JointIsLimitEnabled / EnableLimit */
#define F2D_JP_LOWER 11				/* ...GetLowerLimit; set: SetLimits(value, value2) */
#define F2D_JP_UPPER 12				/* ...GetUpperLimit */
#define F2D_JP_MOTOR_ENABLED 13		/* ...IsMotorEnabled / EnableMotor */
#define F2D_JP_MOTOR_SPEED 14		/* ...Get/SetMotorSpeed */
#define F2D_JP_MAX_MOTOR 15			/* ...Get/SetMaxMotorTorque (revolute, wheel) / Force (prismatic, distance) */
#define F2D_JP_MOTOR_EFFORT 16		/* ...GetMotorTorque / GetMotorForce (get) */
#define F2D_JP_LENGTH 17			/* distanceJointGet/SetLength */
#define F2D_JP_MIN_LENGTH 18		/* distanceJointGetMinLength; set: SetLengthRange(value, value2) */
#define F2D_JP_MAX_LENGTH 19		/* distanceJointGetMaxLength */
#define F2D_JP_CURRENT 20			/* distanceJointGetCurrentLength, revoluteJointGetAngle, prismaticJointGetTranslation */
#define F2D_JP_SPEED 21				/* prismaticJointGetSpeed */
#define F2D_JP_LINEAR_HERTZ 22		/* weldJointGet/SetLinearHertz */
#define F2D_JP_LINEAR_DAMPING 23	/* weldJointGet/SetLinearDampingRatio */
#define F2D_JP_ANGULAR_HERTZ 24		/* weldJointGet/SetAngularHertz */
#define F2D_JP_ANGULAR_DAMPING 25	/* weldJointGet/SetAngularDampingRatio */
#define F2D_JP_LINEAR_OFFSET_X 26	/* motorJointGetLinearOffset; set: SetLinearOffset(value, value2) */
#define F2D_JP_LINEAR_OFFSET_Y 27
#define F2D_JP_ANGULAR_OFFSET 28	/* motorJointGet/SetAngularOffset */
#define F2D_JP_MAX_FORCE 29			/* motorJointGet/SetMaxForce, mouseJointGet/SetMaxForce */
#define F2D_JP_MAX_TORQUE 30		/* motorJointGet/SetMaxTorque */
#define F2D_JP_CORRECTION 31		/* motorJointGet/SetCorrectionFactor */
#define F2D_JP_TARGET_X 32			/* mouseJointGetTarget (set: f2d_mouse_joint_set_target) */
#define F2D_JP_TARGET_Y 33
F2D_API double f2d_joint_get_param( int32_t index1, int32_t worldAndGeneration, int32_t code );
F2D_API void f2d_joint_set_param( int32_t index1, int32_t worldAndGeneration, int32_t code, double value,
								  double value2 );
/* RawBox2D.jointGetBodyA / jointGetBodyB (raw_box2d.dart:723-726): edge 0
 * or 1. */
F2D_API int32_t f2d_joint_get_body( int32_t index1, int32_t worldAndGeneration, int32_t edge, int32_t* bodyIndex1,
									int32_t* bodyWorldAndGeneration );
/* RawBox2D.jointWakeBodies (raw_box2d.dart:745 -> b2Joint_WakeBodies). */
F2D_API void f2d_joint_wake_bodies( int32_t index1, int32_t worldAndGeneration );

/* ---- events (RawBox2D.worldGetContactEvents / worldGetBodyEvents,
 *      raw_box2d_ffi.dart:2172 and :2259) ----------------------------------
 * Counts of the last step's events: begin, end, hit, body move. */
F2D_API void f2d_world_get_event_counts( int32_t worldId, int32_t* counts4 );
/* Begin / end touch events as shape id pairs (index1, worldAndGeneration) x 2
 * = 4 ints per event. Return the number written. */
F2D_API int32_t f2d_world_get_begin_events( int32_t worldId, int32_t* out4, int32_t capacity );
/* The manifold each begin event carries (RawContactBeginEvent normal and
 * points, raw_box2d_ffi.dart:2205-2228; b2ContactBeginTouchEvent.manifold,
 * world.c:630-640), in the order of f2d_world_get_begin_events: 9 floats per
 * event -- normal x, y, point count, then per point (two slots, zero past
 * the count) the world point x, y and the separation. Returns the number
 * written. */
F2D_API int32_t f2d_world_get_begin_manifolds( int32_t worldId, float* out9, int32_t capacity );
/* RawBox2D.worldGetSensorEvents (raw_box2d.dart:1295 -> b2World_GetSensorEvents, world.c:1505):
 * begin and end events of the last step, four ints each (sensor index1,
 * worldAndGeneration, visitor index1, worldAndGeneration); returns the begin
 * count, the end count in *endCount. */
/* User callbacks (b2CustomFilterFcn / b2PreSolveFcn, types.h:1180-1195; forge2d
 * passes them as NativeCallable.isolateLocal, raw_box2d_ffi.dart:2467-2527).
 * Shape ids are (index1, worldAndGeneration) pairs. The custom filter sees
 * every new pair that passed the shape and joint filters (broad_phase.c:
 * 267-278) and every static candidate of continuous collision (solver.c:
 * 270-280): zero keeps the pair apart. The pre-solve callback sees each
 * awake touching contact with pre-solve events and its new manifold, anchors
 * relative to the body origins (contact.c:504-517): zero disables the
 * contact for this step. Both run on the thread that calls f2d_world_step,
 * which then returns only after the step's last callback; the world steps
 * without its CUDA graph while either is set. NULL removes a callback. */
typedef struct f2d_manifold_point_view
{
	float pointX, pointY, anchorAX, anchorAY, anchorBX, anchorBY, separation;
	int32_t id;
} f2d_manifold_point_view;
typedef struct f2d_manifold_view
{
	float normalX, normalY;
	int32_t pointCount, pad0;
	f2d_manifold_point_view points[2];
} f2d_manifold_view;
typedef int32_t ( *f2d_custom_filter_fn )( int32_t shapeAIndex1, int32_t shapeAWorldAndGeneration,
										   int32_t shapeBIndex1, int32_t shapeBWorldAndGeneration, void* context );
typedef int32_t ( *f2d_pre_solve_fn )( int32_t shapeAIndex1, int32_t shapeAWorldAndGeneration,
									   int32_t shapeBIndex1, int32_t shapeBWorldAndGeneration,
									   const f2d_manifold_view* manifold, void* context );
/* RawBox2D.worldSetCustomFilterCallback / worldSetPreSolveCallback (raw_box2d.dart:1358, 1373;
 * the Dart pre-solve callback takes the normal of this view) -> b2World_SetCustomFilterCallback /
 * b2World_SetPreSolveCallback. */
F2D_API void f2d_world_set_custom_filter( int32_t worldId, f2d_custom_filter_fn fn, void* context );
/* RawBox2D.worldExplode (raw_box2d.dart:1342 -> b2World_Explode, world.c:2718):
 * radial impulse on the dynamic shapes within radius + falloff of the
 * position (category against maskBits), waking their bodies. */
/* RawBox2D.worldCastRay (raw_box2d.dart:1318 -> b2World_CastRay, world.c:2222):
 * the callback gets each hit (shape id pair, point, normal, fraction) in
 * ascending fraction and returns -1 (ignore), 0 (stop), a fraction (clip)
 * or 1 (go on). Returns the number of calls. */
typedef float ( *f2d_cast_result_fn )( int32_t shapeIndex1, int32_t shapeWorldAndGeneration, float pointX, float pointY,
									   float normalX, float normalY, float fraction, void* context );
F2D_API int32_t f2d_world_cast_ray( int32_t worldId, double originX, double originY, double translationX,
									double translationY, int64_t categoryBits, int64_t maskBits, f2d_cast_result_fn fn,
									void* context );
F2D_API void f2d_world_explode( int32_t worldId, int64_t maskBits, double positionX, double positionY, double radius,
								double falloff, double impulsePerLength );
F2D_API void f2d_world_set_pre_solve( int32_t worldId, f2d_pre_solve_fn fn, void* context );
F2D_API int32_t f2d_world_get_sensor_events( int32_t worldId, int32_t* begin4, int32_t* end4, int32_t capacity,
											 int32_t* endCount );
F2D_API int32_t f2d_world_get_end_events( int32_t worldId, int32_t* out4, int32_t capacity );
/* Hit events: 4 ints (shape ids) and 5 floats (point.xy normal.xy approachSpeed). */
F2D_API int32_t f2d_world_get_hit_events( int32_t worldId, int32_t* ints4, float* floats5, int32_t capacity );
/* Body move events: 2 ints (body index1, worldAndGeneration) + 1 int fellAsleep,
 * and 4 floats (transform p.xy q.cs) per moved body. */
F2D_API int32_t f2d_world_get_body_events( int32_t worldId, int32_t* ints3, float* floats4, int32_t capacity );

/* ---- queries (RawBox2D.worldCastRayClosest / worldOverlapAabb,
 *      raw_box2d_ffi.dart:2285 and :2388) --------------------------------- */
/* Returns 1 on hit; writes shape id (2 ints) and point.xy normal.xy fraction. */
F2D_API int32_t f2d_world_cast_ray_closest( int32_t worldId, double originX, double originY, double translationX,
											double translationY, int64_t categoryBits, int64_t maskBits,
											int32_t* shape2, float* out5 );
/* Shapes whose fat AABB overlaps the box (b2World_OverlapAABB tests tree
 * boxes only, dynamic_tree.c:1114). Writes shape id pairs; returns the total
 * count (may exceed capacity). */
F2D_API int32_t f2d_world_overlap_aabb( int32_t worldId, double lowerX, double lowerY, double upperX, double upperY,
										int64_t categoryBits, int64_t maskBits, int32_t* shapes2, int32_t capacity );

/* Allocation-free variant of f2d_world_overlap_aabb. It has no reference
 * counterpart: Box2D's b2World_OverlapAABB walks its trees on the CPU and
 * needs no scratch. Same arguments, result order (ascending shape id) and
 * return value as f2d_world_overlap_aabb, but the device scratch is a
 * file-scope __device__ array sized for F2D_OVERLAP_NOALLOC_MAX_SHAPES
 * shapes, and the call makes no cudaMalloc / cudaFree or any other device or
 * host allocation. The first call on each device resolves that array's
 * address with cudaGetSymbolAddress and caches it; make that first call
 * before capturing any stream. Calls that overlap in time on one device
 * share the array and race; serialise them.
 * Returns F2D_NOALLOC_TOO_MANY_SHAPES when the world holds more shapes than
 * the array can take, F2D_NOALLOC_NEEDS_GROWTH when the world's pending
 * uploads would allocate (bodies or shapes created past its device
 * capacities, a sensor shape created, a broadphase tree whose node pool
 * grew, since the last step: step the world, or call f2d_world_reserve
 * first), F2D_NOALLOC_DEVICE_SETUP when the array's address cannot be
 * resolved. No output is written in those cases. */
#define F2D_OVERLAP_NOALLOC_MAX_SHAPES 262144
#define F2D_NOALLOC_TOO_MANY_SHAPES ( -1 )
#define F2D_NOALLOC_NEEDS_GROWTH ( -2 )
#define F2D_NOALLOC_DEVICE_SETUP ( -3 )
F2D_API int32_t f2d_world_overlap_aabb_noalloc( int32_t worldId, double lowerX, double lowerY, double upperX,
												double upperY, int64_t categoryBits, int64_t maskBits,
												int32_t* shapes2, int32_t capacity );

/* ---- bulk state access (for batch readers and parity checks) ------------ */
/* Per body id, 12 floats: p.xy q.cs v.xy w centre.xy valid type sleepTime. */
F2D_API int32_t f2d_world_body_capacity( int32_t worldId );
F2D_API int32_t f2d_world_get_bodies( int32_t worldId, float* out12, int32_t capacity );
/* Per live contact: 9 ints (id shapeA shapeB colour pointCount flags simFlags
 * id0 id1) and 25 floats (normal.xy rollingImpulse, then per point anchorA.xy
 * anchorB.xy point.xy separation normalImpulse tangentImpulse
 * totalNormalImpulse normalVelocity). */
F2D_API int32_t f2d_world_contact_capacity( int32_t worldId );
F2D_API int32_t f2d_world_get_contacts( int32_t worldId, int32_t* ints9, float* floats25, int32_t capacity );
/* Per shape id: aabb(4) fat aabb(4) floats; proxyKey bodyId type flags ints. */
F2D_API int32_t f2d_world_shape_capacity( int32_t worldId );
F2D_API int32_t f2d_world_get_shapes( int32_t worldId, float* floats8, int32_t* ints4, int32_t capacity );
/* Per body id: mass inertia invMass invInertia localCenter.xy minExtent maxExtent. */
F2D_API int32_t f2d_world_get_mass( int32_t worldId, float* out8, int32_t capacity );
/* Colour occupancy (contacts + joints per graph colour, 12 ints; b2Counters.colorCounts). */
F2D_API void f2d_world_get_color_counts( int32_t worldId, int32_t* out12 );
/* Contact ids for the pairs the next step creates (parity with an external
 * Box2D run): rows of (contactId, shapeIdA, shapeIdB), 0-based ids. */
F2D_API void f2d_world_set_contact_plan( int32_t worldId, const int32_t* rows3, int32_t count );
/* Device timing of the last step in milliseconds (CUDA events around the
 * step's launches); 0 before the first step. */
F2D_API double f2d_world_last_step_ms( int32_t worldId );
/* Number of kernel launches the last step enqueued. */
F2D_API int32_t f2d_world_last_step_launches( int32_t worldId );
/* Profiling mode: steps are enqueued without the CUDA graph and with CUDA
 * events between phases (b2Profile's per-stage timers, types.h:466-490). */
F2D_API void f2d_world_set_profiling( int32_t worldId, int32_t enabled );
/* Last profiled step, ms: broadphase, narrowphase, colouring, solver set-up,
 * solver kernel, finalize. */
F2D_API void f2d_world_get_phase_ms( int32_t worldId, double* out6 );
/* Last profiled step, ms: the partial rebuild of the dynamic and kinematic
 * trees, which runs on a second stream beside the narrowphase and the
 * colouring (world.c:488-502). */
F2D_API double f2d_world_get_rebuild_ms( int32_t worldId );
/* awake bodies, live contacts, touching contacts, overflow contacts, active
 * colours, colouring rounds, shapes, joints (b2Counters, types.h:493-506). */
F2D_API void f2d_world_get_counters( int32_t worldId, int32_t* out8 );
/* The grid barriers the last grid-wide solver launch passed (out2[0]; 0 after
 * a step on the cluster solver) and, when probeBarriers > 0, the measured
 * microseconds per grid barrier on that solver's grid (out2[1]): the latency
 * floor of the solver kernel is their product. */
F2D_API void f2d_world_get_solver_latency( int32_t worldId, int32_t probeBarriers, double* out2 );
/* ---- learned warm start (no reference counterpart) ----------------------
 * A small MLP [12 -> 64 -> 64 -> 2] (BF16 weights, FP32 accumulation,
 * tensor-core MMA) predicts the normal and tangent impulses of manifold
 * points that have no cached impulse; persisting points keep Box2D's cached
 * impulses and every solver iteration still runs. Features per new point:
 * normal.xy, normal and tangent relative velocity, separation, anchorA and
 * anchorB along the tangent and the normal, the effective normal and
 * tangent masses (from the inverse masses and inertias), friction. A sample
 * is the 12 features plus the normal and tangent impulse the plain solver
 * ended the step with. */
/* Record up to `capacity` samples from the following steps (0 stops). */
F2D_API void f2d_world_set_sample_recording( int32_t worldId, int32_t capacity );
F2D_API int32_t f2d_world_sample_count( int32_t worldId );
/* Copies recorded samples (14 floats each); returns the number written. */
F2D_API int32_t f2d_world_get_samples( int32_t worldId, float* out14, int32_t capacity );
/* Predict warm-start impulses of new points with `model` (0 disables). */
F2D_API int32_t f2d_world_set_warm_start_model( int32_t worldId, int32_t model );
/* Model handle (> 0), He-uniform weights from seed; 0 on failure. */
F2D_API int32_t f2d_mlp_create( uint32_t seed );
F2D_API void f2d_mlp_destroy( int32_t model );
/* FP32 master parameters: W1 [64][16] (columns 12..15 zero), W2 [64][64],
 * W3 [8][64] (rows 2..7 zero), b1 [64], b2 [64], b3 [8]. */
F2D_API int32_t f2d_mlp_param_count( void );
F2D_API void f2d_mlp_get_params( int32_t model, float* out );
F2D_API void f2d_mlp_set_params( int32_t model, const float* in );
/* Per-column mean and 1/std of the 12 features and 2 targets. */
F2D_API void f2d_mlp_set_normalization( int32_t model, const float* mean14, const float* invStd14 );
/* Gradient of 0.5 * mean ||y - t||^2 (normalised units) over n samples at
 * the current parameters, no update; returns the loss. */
F2D_API float f2d_mlp_gradient( int32_t model, const float* samples14, int32_t n, float* grad );
/* Adam training on the GPU; returns the mean loss of the last epoch. */
F2D_API float f2d_mlp_train( int32_t model, const float* samples14, int32_t n, int32_t epochs, int32_t batch,
							 float learningRate, uint32_t seed );
/* Predicted (normal, tangent) impulses of n raw feature rows. */
F2D_API void f2d_mlp_predict( int32_t model, const float* feats12, int32_t n, float* out2 );

/* Autotuner (no reference counterpart). Steps the world through every
 * candidate launch configuration -- solver kernel shape (1 thread-block
 * cluster when the bodies fit, grid-wide with 512- or 256-thread blocks) x
 * broadphase leaf-order refresh period (4, 8, 16, 32 steps) -- timing each
 * over max(stepsPerCandidate, period) steps, and keeps the fastest. The
 * tuning steps are ordinary steps of the world; no configuration changes any
 * result. chosen3 (optional) receives {solver variant, period, steps
 * taken}. Returns the accumulated F2D_STATUS_* bits. */
F2D_API int32_t f2d_world_autotune( int32_t worldId, double timeStep, int32_t subStepCount,
									int32_t stepsPerCandidate, int32_t* chosen3 );
/* Current {solver variant, leaf-order period} (0 = defaults). */
F2D_API void f2d_world_get_tuning( int32_t worldId, int32_t* out2 );
/* Capacities chosen at creation can be raised before the first step. */
F2D_API void f2d_world_reserve( int32_t worldId, int32_t bodies, int32_t shapes, int32_t contacts, int32_t joints );

#ifdef __cplusplus
}
#endif

#endif
