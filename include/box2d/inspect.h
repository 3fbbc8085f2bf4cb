/*
 * box2d/inspect.h -- read-only introspection of a world's step-path state.
 *
 * Has no counterpart in the reference API.  It exposes what the reference keeps in
 * private structs (contact ids and shape pairs from src/contact.h:50-79, colour and
 * local index from src/constraint_graph.c:64-214, manifolds and accumulated impulses
 * from include/box2d/collision.h:474-520, fat AABBs and broadphase proxy keys from
 * src/shape.h:14-60) so that pair sets, colour assignments, manifolds and body state
 * can be compared bit for bit between two implementations of b2World_Step.
 *
 * Include box2d/box2d.h (or any header that defines b2WorldId) before this one.
 */
#ifndef B2_INSPECT_H
#define B2_INSPECT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Floats per body written by b2World_InspectBodies: p.x p.y q.c q.s v.x v.y w type. */
#define B2_INSPECT_BODY_FLOATS 8

typedef struct b2InspectPoint
{
	float anchorA[2];
	float anchorB[2];
	float point[2];
	float separation;
	float normalImpulse;
	float tangentImpulse;
	float maxNormalImpulse;
	float normalVelocity;
	int32_t id;
	int32_t persisted;
} b2InspectPoint;

typedef struct b2InspectContact
{
	int32_t contactId;
	int32_t shapeIdA;
	int32_t shapeIdB;
	int32_t colorIndex; /* -1 when not in the constraint graph */
	int32_t localIndex; /* index inside its colour array or the non-touching array */
	int32_t touching;	/* 1 when the solid shapes touch */
	int32_t pointCount;
	float normal[2];
	float friction;
	float restitution;
	b2InspectPoint points[2];
} b2InspectContact;

typedef struct b2InspectShape
{
	float aabb[4];	  /* lower.x lower.y upper.x upper.y */
	float fatAABB[4]; /* the broadphase proxy box */
	int32_t proxyKey; /* (proxy id << 2) | body type, -1 if none */
	int32_t bodyId;
} b2InspectShape;

/* Each returns the number of records available; writes at most `capacity` of them.
 * Bodies and shapes are indexed by their zero-based id (index1 - 1); free slots are
 * written with a NaN position (bodies) or proxyKey -1 (shapes).  Contacts are written
 * in ascending contact id order. */
int b2World_InspectBodies( b2WorldId worldId, float* out, int capacity );
int b2World_InspectShapes( b2WorldId worldId, b2InspectShape* out, int capacity );
int b2World_InspectContacts( b2WorldId worldId, b2InspectContact* out, int capacity );

/* Two ints per body id: the solver set (0 static, 2 awake, 3 and up a sleeping set; the
 * reference's src/solver_set.h:11-30 numbering) and the island id (-1 for none), both
 * -1 for a free slot.  Set and island ids come from id pools, so two implementations
 * that move islands between sets in the same order agree on them exactly. */
int b2World_InspectIslands( b2WorldId worldId, int* out, int capacity );

#ifdef __cplusplus
}
#endif

#endif
