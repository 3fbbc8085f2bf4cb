/*
 * ref_probe.c -- introspection shim compiled together with the reference sources.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile.ref into oracle/_ref/ next to the
 * unmodified reference library so that tests can read the reference's private step
 * state (pairs, colours, manifolds, proxies) through the b2World_Inspect* functions of
 * include/box2d/inspect.h.  It reads the reference's internal structs through the
 * reference's own internal headers (src/world.h:47-163, src/contact.h:50-141,
 * src/shape.h:14-60, src/body.h:16-133) and never changes them.
 */
#include "body.h"
#include "contact.h"
#include "shape.h"
#include "solver_set.h"
#include "world.h"

#include "box2d/box2d.h"

#include B2_INSPECT_HEADER

#include <math.h>
#include <string.h>

int b2World_InspectBodies( b2WorldId worldId, float* out, int capacity )
{
	b2World* world = b2GetWorldFromId( worldId );
	int count = b2Array( world->bodyArray ).count;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		float* o = out + B2_INSPECT_BODY_FLOATS * i;
		b2Body* body = world->bodyArray + i;
		if ( body->id != i || body->setIndex == B2_NULL_INDEX )
		{
			for ( int k = 0; k < B2_INSPECT_BODY_FLOATS; ++k )
				o[k] = NAN;
			continue;
		}
		b2Transform xf = b2GetBodyTransformQuick( world, body );
		b2BodyState* state = b2GetBodyState( world, body );
		o[0] = xf.p.x;
		o[1] = xf.p.y;
		o[2] = xf.q.c;
		o[3] = xf.q.s;
		o[4] = state ? state->linearVelocity.x : 0.0f;
		o[5] = state ? state->linearVelocity.y : 0.0f;
		o[6] = state ? state->angularVelocity : 0.0f;
		o[7] = (float)body->type;
	}
	return count;
}

int b2World_InspectIslands( b2WorldId worldId, int* out, int capacity )
{
	b2World* world = b2GetWorldFromId( worldId );
	int count = b2Array( world->bodyArray ).count;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		b2Body* body = world->bodyArray + i;
		bool live = body->id == i && body->setIndex != B2_NULL_INDEX;
		out[2 * i] = live ? body->setIndex : -1;
		out[2 * i + 1] = live ? body->islandId : -1;
	}
	return count;
}

int b2World_InspectShapes( b2WorldId worldId, b2InspectShape* out, int capacity )
{
	b2World* world = b2GetWorldFromId( worldId );
	int count = b2Array( world->shapeArray ).count;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		b2Shape* shape = world->shapeArray + i;
		b2InspectShape* o = out + i;
		memset( o, 0, sizeof( *o ) );
		if ( shape->id != i )
		{
			o->proxyKey = -1;
			o->bodyId = -1;
			continue;
		}
		o->aabb[0] = shape->aabb.lowerBound.x;
		o->aabb[1] = shape->aabb.lowerBound.y;
		o->aabb[2] = shape->aabb.upperBound.x;
		o->aabb[3] = shape->aabb.upperBound.y;
		o->fatAABB[0] = shape->fatAABB.lowerBound.x;
		o->fatAABB[1] = shape->fatAABB.lowerBound.y;
		o->fatAABB[2] = shape->fatAABB.upperBound.x;
		o->fatAABB[3] = shape->fatAABB.upperBound.y;
		o->proxyKey = shape->proxyKey;
		o->bodyId = shape->bodyId;
	}
	return count;
}

int b2World_InspectContacts( b2WorldId worldId, b2InspectContact* out, int capacity )
{
	b2World* world = b2GetWorldFromId( worldId );
	int idCount = b2Array( world->contactArray ).count;
	int n = 0;
	for ( int i = 0; i < idCount; ++i )
	{
		b2Contact* contact = world->contactArray + i;
		if ( contact->contactId != i || contact->setIndex == B2_NULL_INDEX )
			continue;
		if ( n < capacity )
		{
			b2ContactSim* sim = b2GetContactSim( world, contact );
			b2InspectContact* o = out + n;
			memset( o, 0, sizeof( *o ) );
			o->contactId = i;
			o->shapeIdA = contact->shapeIdA;
			o->shapeIdB = contact->shapeIdB;
			o->colorIndex = contact->colorIndex;
			o->localIndex = contact->localIndex;
			o->touching = ( contact->flags & b2_contactTouchingFlag ) ? 1 : 0;
			o->pointCount = sim->manifold.pointCount;
			o->normal[0] = sim->manifold.normal.x;
			o->normal[1] = sim->manifold.normal.y;
			o->friction = sim->friction;
			o->restitution = sim->restitution;
			for ( int k = 0; k < 2; ++k )
			{
				b2ManifoldPoint* mp = sim->manifold.points + k;
				b2InspectPoint* p = o->points + k;
				p->anchorA[0] = mp->anchorA.x;
				p->anchorA[1] = mp->anchorA.y;
				p->anchorB[0] = mp->anchorB.x;
				p->anchorB[1] = mp->anchorB.y;
				p->point[0] = mp->point.x;
				p->point[1] = mp->point.y;
				p->separation = mp->separation;
				p->normalImpulse = mp->normalImpulse;
				p->tangentImpulse = mp->tangentImpulse;
				p->maxNormalImpulse = mp->maxNormalImpulse;
				p->normalVelocity = mp->normalVelocity;
				p->id = mp->id;
				p->persisted = mp->persisted ? 1 : 0;
			}
		}
		n += 1;
	}
	return n;
}
