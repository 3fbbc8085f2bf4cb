/*
 * b2o_inspect.c -- introspection entry points of the plain-C oracle
 * (TEST INFRASTRUCTURE), same contract as include/box2d/inspect.h.
 */
#include "b2o.h"

#include "box2d/inspect.h"

#include <string.h>

int b2World_InspectBodies( b2WorldId worldId, float* out, int capacity )
{
	oWorld* w = o_world( worldId );
	int count = w->bodyIds.next;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		float* o = out + B2_INSPECT_BODY_FLOATS * i;
		oBody* b = w->bodies + i;
		if ( b->id != i )
		{
			for ( int k = 0; k < B2_INSPECT_BODY_FLOATS; ++k )
				o[k] = NAN;
			continue;
		}
		o[0] = (float)b->xf.p.x;
		o[1] = (float)b->xf.p.y;
		o[2] = (float)b->xf.q.c;
		o[3] = (float)b->xf.q.s;
		/* velocities live in the awake set only */
		bool awake = b->setIndex == O_SET_AWAKE;
		o[4] = awake ? (float)b->v.x : 0.0f;
		o[5] = awake ? (float)b->v.y : 0.0f;
		o[6] = awake ? (float)b->w : 0.0f;
		o[7] = (float)b->type;
	}
	return count;
}

int b2World_InspectIslands( b2WorldId worldId, int* out, int capacity )
{
	oWorld* w = o_world( worldId );
	int count = w->bodyIds.next;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		oBody* b = w->bodies + i;
		out[2 * i] = b->id == i ? b->setIndex : -1;
		out[2 * i + 1] = b->id == i ? b->islandId : -1;
	}
	return count;
}

int b2World_InspectShapes( b2WorldId worldId, b2InspectShape* out, int capacity )
{
	oWorld* w = o_world( worldId );
	int count = w->shapeIds.next;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		oShape* s = w->shapes + i;
		b2InspectShape* o = out + i;
		memset( o, 0, sizeof( *o ) );
		if ( s->id != i )
		{
			o->proxyKey = -1;
			o->bodyId = -1;
			continue;
		}
		o->aabb[0] = (float)s->aabb.lo.x;
		o->aabb[1] = (float)s->aabb.lo.y;
		o->aabb[2] = (float)s->aabb.hi.x;
		o->aabb[3] = (float)s->aabb.hi.y;
		o->fatAABB[0] = (float)s->fatAABB.lo.x;
		o->fatAABB[1] = (float)s->fatAABB.lo.y;
		o->fatAABB[2] = (float)s->fatAABB.hi.x;
		o->fatAABB[3] = (float)s->fatAABB.hi.y;
		o->proxyKey = s->proxyKey;
		o->bodyId = s->bodyId;
	}
	return count;
}

int b2World_InspectContacts( b2WorldId worldId, b2InspectContact* out, int capacity )
{
	oWorld* w = o_world( worldId );
	int n = 0;
	for ( int i = 0; i < w->contactIds.next; ++i )
	{
		oContact* c = w->contacts + i;
		if ( c->id != i )
			continue;
		if ( n < capacity )
		{
			b2InspectContact* o = out + n;
			memset( o, 0, sizeof( *o ) );
			o->contactId = i;
			o->shapeIdA = c->shapeIdA;
			o->shapeIdB = c->shapeIdB;
			o->colorIndex = c->colorIndex;
			o->localIndex = c->localIndex;
			o->touching = ( c->flags & OC_TOUCHING ) ? 1 : 0;
			o->pointCount = c->manifold.count;
			o->normal[0] = (float)c->manifold.normal.x;
			o->normal[1] = (float)c->manifold.normal.y;
			o->friction = (float)c->friction;
			o->restitution = (float)c->restitution;
			for ( int k = 0; k < 2; ++k )
			{
				const oMPoint* mp = c->manifold.pts + k;
				b2InspectPoint* p = o->points + k;
				p->anchorA[0] = (float)mp->anchorA.x;
				p->anchorA[1] = (float)mp->anchorA.y;
				p->anchorB[0] = (float)mp->anchorB.x;
				p->anchorB[1] = (float)mp->anchorB.y;
				p->point[0] = (float)mp->point.x;
				p->point[1] = (float)mp->point.y;
				p->separation = (float)mp->separation;
				p->normalImpulse = (float)mp->normalImpulse;
				p->tangentImpulse = (float)mp->tangentImpulse;
				p->maxNormalImpulse = (float)mp->maxNormalImpulse;
				p->normalVelocity = (float)mp->normalVelocity;
				p->id = mp->id;
				p->persisted = mp->persisted ? 1 : 0;
			}
		}
		n += 1;
	}
	return n;
}

/* Oracle-only queries. */
int b2o_ToiEventCount( b2WorldId worldId ) { return o_world( worldId )->toiEvents; }

/* Double-precision state access for the FP64 gradient check (meaningful when the oracle
 * is compiled with -DB2O_F64). out: p.x p.y q.c q.s v.x v.y w per body id. */
int b2o_GetBodyStateF64( b2WorldId worldId, double* out, int capacity )
{
	oWorld* w = o_world( worldId );
	int count = w->bodyIds.next;
	for ( int i = 0; i < count && i < capacity; ++i )
	{
		oBody* b = w->bodies + i;
		double* o = out + 7 * i;
		o[0] = (double)b->xf.p.x;
		o[1] = (double)b->xf.p.y;
		o[2] = (double)b->xf.q.c;
		o[3] = (double)b->xf.q.s;
		o[4] = (double)b->v.x;
		o[5] = (double)b->v.y;
		o[6] = (double)b->w;
	}
	return count;
}

void b2o_SetBodyVelocityF64( b2WorldId worldId, int bodyIndex, double vx, double vy, double w )
{
	oBody* b = o_world( worldId )->bodies + bodyIndex;
	b->v.x = (b2r)vx;
	b->v.y = (b2r)vy;
	b->w = (b2r)w;
}

void b2o_SetShapeFrictionF64( b2WorldId worldId, int shapeIndex, double friction )
{
	o_world( worldId )->shapes[shapeIndex].friction = (b2r)friction;
}
