/*
 * box2d/collision.h -- geometry, mass, AABB and contact-manifold types and functions.
 *
 * Shape and manifold structs keep the exact layout of the reference
 * `include/box2d/collision.h:38-520` so that geometry built by a caller (b2MakeBox,
 * b2Polygon literals) and manifolds returned to a caller cross the C ABI unchanged.
 * The manifold functions declared here run on the host in this library; the same
 * arithmetic runs in the device narrowphase kernel (one shared source).
 */
#pragma once

#include "base.h"
#include "math_functions.h"

#include <stdbool.h>

#define b2_maxPolygonVertices 8

typedef struct b2RayCastInput
{
	b2Vec2 origin;
	b2Vec2 translation;
	float maxFraction;
} b2RayCastInput;

typedef struct b2CastOutput
{
	b2Vec2 normal;
	b2Vec2 point;
	float fraction;
	int32_t iterations;
	bool hit;
} b2CastOutput;

typedef struct b2MassData
{
	float mass;
	b2Vec2 center;
	float rotationalInertia;
} b2MassData;

typedef struct b2Circle
{
	b2Vec2 center;
	float radius;
} b2Circle;

typedef struct b2Capsule
{
	b2Vec2 center1;
	b2Vec2 center2;
	float radius;
} b2Capsule;

/* Convex polygon with counter-clockwise vertices and outward unit edge normals. */
typedef struct b2Polygon
{
	b2Vec2 vertices[b2_maxPolygonVertices];
	b2Vec2 normals[b2_maxPolygonVertices];
	b2Vec2 centroid;
	float radius;
	int32_t count;
} b2Polygon;

typedef struct b2Segment
{
	b2Vec2 point1;
	b2Vec2 point2;
} b2Segment;

typedef struct b2SmoothSegment
{
	b2Vec2 ghost1;
	b2Segment segment;
	b2Vec2 ghost2;
	int32_t chainId;
} b2SmoothSegment;

typedef struct b2Hull
{
	b2Vec2 points[b2_maxPolygonVertices];
	int32_t count;
} b2Hull;

B2_API b2Polygon b2MakeSquare( float h );
B2_API b2Polygon b2MakeBox( float hx, float hy );
B2_API b2Polygon b2MakeRoundedBox( float hx, float hy, float radius );
B2_API b2Polygon b2MakeOffsetBox( float hx, float hy, b2Vec2 center, float angle );
B2_API b2Polygon b2TransformPolygon( b2Transform transform, const b2Polygon* polygon );

B2_API b2MassData b2ComputeCircleMass( const b2Circle* shape, float density );
B2_API b2MassData b2ComputeCapsuleMass( const b2Capsule* shape, float density );
B2_API b2MassData b2ComputePolygonMass( const b2Polygon* shape, float density );

B2_API b2AABB b2ComputeCircleAABB( const b2Circle* shape, b2Transform transform );
B2_API b2AABB b2ComputeCapsuleAABB( const b2Capsule* shape, b2Transform transform );
B2_API b2AABB b2ComputePolygonAABB( const b2Polygon* shape, b2Transform transform );
B2_API b2AABB b2ComputeSegmentAABB( const b2Segment* shape, b2Transform transform );

typedef struct b2SegmentDistanceResult
{
	b2Vec2 closest1;
	b2Vec2 closest2;
	float fraction1;
	float fraction2;
	float distanceSquared;
} b2SegmentDistanceResult;

/* Closest points of two segments (reference src/distance.c:32-107). */
B2_API b2SegmentDistanceResult b2SegmentDistance( b2Vec2 p1, b2Vec2 q1, b2Vec2 p2, b2Vec2 q2 );

/* GJK warm-start cache carried by each contact (reference collision.h:300-306). */
typedef struct b2DistanceCache
{
	uint16_t count;
	uint8_t indexA[3];
	uint8_t indexB[3];
} b2DistanceCache;

static const b2DistanceCache b2_emptyDistanceCache = B2_ZERO_INIT;

typedef struct b2ManifoldPoint
{
	b2Vec2 point;
	b2Vec2 anchorA;
	b2Vec2 anchorB;
	float separation;
	float normalImpulse;
	float tangentImpulse;
	float maxNormalImpulse;
	float normalVelocity;
	uint16_t id;
	bool persisted;
} b2ManifoldPoint;

typedef struct b2Manifold
{
	b2ManifoldPoint points[2];
	b2Vec2 normal;
	int32_t pointCount;
} b2Manifold;

B2_API b2Manifold b2CollideCircles( const b2Circle* circleA, b2Transform xfA, const b2Circle* circleB, b2Transform xfB );
B2_API b2Manifold b2CollideCapsuleAndCircle( const b2Capsule* capsuleA, b2Transform xfA, const b2Circle* circleB,
											 b2Transform xfB );
B2_API b2Manifold b2CollideSegmentAndCircle( const b2Segment* segmentA, b2Transform xfA, const b2Circle* circleB,
											 b2Transform xfB );
B2_API b2Manifold b2CollidePolygonAndCircle( const b2Polygon* polygonA, b2Transform xfA, const b2Circle* circleB,
											 b2Transform xfB );
B2_API b2Manifold b2CollideCapsules( const b2Capsule* capsuleA, b2Transform xfA, const b2Capsule* capsuleB, b2Transform xfB );
B2_API b2Manifold b2CollideSegmentAndCapsule( const b2Segment* segmentA, b2Transform xfA, const b2Capsule* capsuleB,
											  b2Transform xfB );
B2_API b2Manifold b2CollidePolygonAndCapsule( const b2Polygon* polygonA, b2Transform xfA, const b2Capsule* capsuleB,
											  b2Transform xfB );
B2_API b2Manifold b2CollidePolygons( const b2Polygon* polygonA, b2Transform xfA, const b2Polygon* polygonB, b2Transform xfB );
B2_API b2Manifold b2CollideSegmentAndPolygon( const b2Segment* segmentA, b2Transform xfA, const b2Polygon* polygonB,
											  b2Transform xfB );
/* Chain links (reference collision.h:557-567): one-sided, with ghost vertices; the
 * capsule and polygon forms warm-start from and update the caller's distance cache. */
B2_API b2Manifold b2CollideSmoothSegmentAndCircle( const b2SmoothSegment* smoothSegmentA, b2Transform xfA,
												   const b2Circle* circleB, b2Transform xfB );
B2_API b2Manifold b2CollideSmoothSegmentAndCapsule( const b2SmoothSegment* smoothSegmentA, b2Transform xfA,
													const b2Capsule* capsuleB, b2Transform xfB, b2DistanceCache* cache );
B2_API b2Manifold b2CollideSmoothSegmentAndPolygon( const b2SmoothSegment* smoothSegmentA, b2Transform xfA,
													const b2Polygon* polygonB, b2Transform xfB, b2DistanceCache* cache );

#define b2_defaultCategoryBits ( 0x00000001 )
#define b2_defaultMaskBits ( 0xFFFFFFFF )
