/*
 * b2o_solver.c -- soft-step solver, body finalisation, proxy enlargement
 * and the fast-body path of the plain-C oracle (TEST INFRASTRUCTURE).
 *
 * Restates the reference: step context and softness (src/world.c:717-745,
 * src/solver.h:144-156); b2Solve stage order (src/solver.c:559-731, :1108-1668);
 * velocity / position integration (:34-93, :146-163); finalisation (:165-351); proxy
 * enlargement (:1741-1797); the fast-body part of continuous collision (:787-1105,
 * :1807-1954).  Contact constraints follow src/contact_solver.c: the overflow colour
 * uses the scalar path (:21-471) and graph colours the 8-lane path (:597-1293), whose
 * arithmetic differs; both are restated lane by lane, including the dummy second point
 * the 8-lane path evaluates for one-point manifolds.  Joints of every type are in
 * b2o_joint.c.
 */
#include "b2o.h"

#include <string.h>

void o_capture_inputs( oWorld* w );
void o_capture_outputs( oWorld* w );

oSoft o_make_soft( b2r hertz, b2r zeta, b2r h )
{
	oSoft s;
	if ( hertz == R( 0 ) )
	{
		s.biasRate = 0;
		s.massScale = 1;
		s.impulseScale = 0;
		return s;
	}
	b2r omega = R( 2 ) * O_PI * hertz;
	b2r a1 = R( 2 ) * zeta + h * omega;
	b2r a2 = h * omega * a1;
	b2r a3 = R( 1 ) / ( R( 1 ) + a2 );
	s.biasRate = omega / a1;
	s.massScale = a2 * a3;
	s.impulseScale = a3;
	return s;
}

/* Body solver state with a detached dummy for static bodies. */
static oState load_state( oWorld* w, int index )
{
	oState s;
	if ( index == O_NULL )
	{
		s.v = ov( 0, 0 );
		s.w = 0;
		s.dp = ov( 0, 0 );
		s.dq = orot( 1, 0 );
		return s;
	}
	oBody* b = w->bodies + index;
	s.v = b->v;
	s.w = b->w;
	s.dp = b->dp;
	s.dq = b->dq;
	return s;
}

static void store_velocity( oWorld* w, int index, oVec v, b2r a )
{
	if ( index == O_NULL )
		return;
	w->bodies[index].v = v;
	w->bodies[index].w = a;
}

/* ------------------------------------------------------------ contact prepare (shared) */
static void prepare_contact( oWorld* w, const oStep* st, oConstraint* k, oContact* c )
{
	const oManifold* m = &c->manifold;
	b2r warm = st->enableWarmStarting ? R( 1 ) : R( 0 );
	k->contactId = c->id;
	k->indexA = c->simIndexA;
	k->indexB = c->simIndexB;
	k->normal = m->normal;
	k->friction = c->friction;
	k->restitution = c->restitution;
	k->pointCount = m->count;
	oState sA = load_state( w, k->indexA );
	oState sB = load_state( w, k->indexB );
	b2r mA = c->invMassA, iA = c->invIA, mB = c->invMassB, iB = c->invIB;
	k->soft = ( k->indexA == O_NULL || k->indexB == O_NULL ) ? st->staticSoft : st->contactSoft;
	k->invMassA = mA;
	k->invIA = iA;
	k->invMassB = mB;
	k->invIB = iB;
	oVec n = k->normal;
	oVec t = oright( n );
	memset( k->pts, 0, sizeof( k->pts ) );
	for ( int j = 0; j < m->count; ++j )
	{
		const oMPoint* mp = m->pts + j;
		oCPoint* cp = k->pts + j;
		cp->normalImpulse = warm * mp->normalImpulse;
		cp->tangentImpulse = warm * mp->tangentImpulse;
		cp->maxNormalImpulse = 0;
		oVec rA = mp->anchorA, rB = mp->anchorB;
		cp->anchorA = rA;
		cp->anchorB = rB;
		cp->baseSeparation = mp->separation - odot( osub( rB, rA ), n );
		b2r rnA = ocross( rA, n ), rnB = ocross( rB, n );
		b2r kN = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
		cp->normalMass = kN > R( 0 ) ? R( 1 ) / kN : R( 0 );
		b2r rtA = ocross( rA, t ), rtB = ocross( rB, t );
		b2r kT = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
		cp->tangentMass = kT > R( 0 ) ? R( 1 ) / kT : R( 0 );
		oVec vrA = oadd( sA.v, ocross_sv( sA.w, rA ) );
		oVec vrB = oadd( sB.v, ocross_sv( sB.w, rB ) );
		cp->relativeVelocity = odot( n, osub( vrB, vrA ) );
	}
}

/* ------------------------------------------------------------ overflow (scalar) path */
static void warm_start_overflow( oWorld* w, oConstraint* k )
{
	oState sA = load_state( w, k->indexA );
	oState sB = load_state( w, k->indexB );
	oVec vA = sA.v, vB = sB.v;
	b2r wA = sA.w, wB = sB.w;
	b2r mA = k->invMassA, iA = k->invIA, mB = k->invMassB, iB = k->invIB;
	oVec n = k->normal, t = oright( n );
	for ( int j = 0; j < k->pointCount; ++j )
	{
		oCPoint* cp = k->pts + j;
		oVec P = oadd( omulsv( cp->normalImpulse, n ), omulsv( cp->tangentImpulse, t ) );
		wA -= iA * ocross( cp->anchorA, P );
		vA = omuladd( vA, -mA, P );
		wB += iB * ocross( cp->anchorB, P );
		vB = omuladd( vB, mB, P );
	}
	store_velocity( w, k->indexA, vA, wA );
	store_velocity( w, k->indexB, vB, wB );
}

static void solve_overflow( oWorld* w, const oStep* st, oConstraint* k, bool useBias )
{
	oState sA = load_state( w, k->indexA );
	oState sB = load_state( w, k->indexB );
	b2r mA = k->invMassA, iA = k->invIA, mB = k->invMassB, iB = k->invIB;
	oVec vA = sA.v, vB = sB.v;
	b2r wA = sA.w, wB = sB.w;
	oRot dqA = sA.dq, dqB = sB.dq;
	oVec dp = osub( sB.dp, sA.dp );
	oVec n = k->normal, t = oright( n );
	b2r friction = k->friction;
	oSoft soft = k->soft;
	for ( int j = 0; j < k->pointCount; ++j )
	{
		oCPoint* cp = k->pts + j;
		oVec ds = oadd( dp, osub( orotate( dqB, cp->anchorB ), orotate( dqA, cp->anchorA ) ) );
		b2r s = odot( ds, n ) + cp->baseSeparation;
		b2r velocityBias = 0, massScale = 1, impulseScale = 0;
		if ( s > R( 0 ) )
			velocityBias = s * st->inv_h;
		else if ( useBias )
		{
			velocityBias = omax( soft.biasRate * s, -st->pushout );
			massScale = soft.massScale;
			impulseScale = soft.impulseScale;
		}
		oVec rA = cp->anchorA, rB = cp->anchorB;
		oVec vrA = oadd( vA, ocross_sv( wA, rA ) );
		oVec vrB = oadd( vB, ocross_sv( wB, rB ) );
		b2r vn = odot( osub( vrB, vrA ), n );
		b2r impulse = -cp->normalMass * massScale * ( vn + velocityBias ) - impulseScale * cp->normalImpulse;
		b2r newImpulse = omax( cp->normalImpulse + impulse, R( 0 ) );
		impulse = newImpulse - cp->normalImpulse;
		cp->normalImpulse = newImpulse;
		cp->maxNormalImpulse = omax( cp->maxNormalImpulse, impulse );
		oVec P = omulsv( impulse, n );
		vA = omulsub( vA, mA, P );
		wA -= iA * ocross( rA, P );
		vB = omuladd( vB, mB, P );
		wB += iB * ocross( rB, P );
	}
	for ( int j = 0; j < k->pointCount; ++j )
	{
		oCPoint* cp = k->pts + j;
		oVec rA = cp->anchorA, rB = cp->anchorB;
		oVec vrB = oadd( vB, ocross_sv( wB, rB ) );
		oVec vrA = oadd( vA, ocross_sv( wA, rA ) );
		b2r vt = odot( osub( vrB, vrA ), t );
		b2r impulse = cp->tangentMass * ( -vt );
		b2r maxFriction = friction * cp->normalImpulse;
		b2r newImpulse = oclamp( cp->tangentImpulse + impulse, -maxFriction, maxFriction );
		impulse = newImpulse - cp->tangentImpulse;
		cp->tangentImpulse = newImpulse;
		oVec P = omulsv( impulse, t );
		vA = omulsub( vA, mA, P );
		wA -= iA * ocross( rA, P );
		vB = omuladd( vB, mB, P );
		wB += iB * ocross( rB, P );
	}
	store_velocity( w, k->indexA, vA, wA );
	store_velocity( w, k->indexB, vB, wB );
}

static void restitution_overflow( oWorld* w, const oStep* st, oConstraint* k )
{
	if ( k->restitution == R( 0 ) )
		return;
	oState sA = load_state( w, k->indexA );
	oState sB = load_state( w, k->indexB );
	b2r mA = k->invMassA, iA = k->invIA, mB = k->invMassB, iB = k->invIB;
	oVec vA = sA.v, vB = sB.v;
	b2r wA = sA.w, wB = sB.w;
	oVec n = k->normal;
	for ( int j = 0; j < k->pointCount; ++j )
	{
		oCPoint* cp = k->pts + j;
		if ( cp->relativeVelocity > -st->restitutionThreshold || cp->maxNormalImpulse == R( 0 ) )
			continue;
		oVec rA = cp->anchorA, rB = cp->anchorB;
		oVec vrB = oadd( vB, ocross_sv( wB, rB ) );
		oVec vrA = oadd( vA, ocross_sv( wA, rA ) );
		b2r vn = odot( osub( vrB, vrA ), n );
		b2r impulse = -cp->normalMass * ( vn + k->restitution * cp->relativeVelocity );
		b2r newImpulse = omax( cp->normalImpulse + impulse, R( 0 ) );
		impulse = newImpulse - cp->normalImpulse;
		cp->normalImpulse = newImpulse;
		cp->maxNormalImpulse = omax( cp->maxNormalImpulse, impulse );
		oVec P = omulsv( impulse, n );
		vA = omulsub( vA, mA, P );
		wA -= iA * ocross( rA, P );
		vB = omuladd( vB, mB, P );
		wB += iB * ocross( rB, P );
	}
	store_velocity( w, k->indexA, vA, wA );
	store_velocity( w, k->indexB, vB, wB );
}

/* ------------------------------------------------------------ graph-colour (8-lane) path */
/* One lane of the 8-wide record: both point slots are always evaluated; a one-point
 * manifold carries zeros in slot 1 exactly like the reference remainder data. */
static void apply_impulse_lane( oVec* vA, b2r* wA, oVec* vB, b2r* wB, const oConstraint* k, oVec rA, oVec rB, b2r Px, b2r Py )
{
	vA->x = vA->x - k->invMassA * Px;
	vA->y = vA->y - k->invMassA * Py;
	*wA = *wA - k->invIA * ( rA.x * Py - rA.y * Px );
	vB->x = vB->x + k->invMassB * Px;
	vB->y = vB->y + k->invMassB * Py;
	*wB = *wB + k->invIB * ( rB.x * Py - rB.y * Px );
}

static void warm_start_lane( oWorld* w, oConstraint* k )
{
	oState sA = load_state( w, k->indexA );
	oState sB = load_state( w, k->indexB );
	b2r tX = k->normal.y;
	b2r tY = R( 0 ) - k->normal.x;
	for ( int j = 0; j < 2; ++j )
	{
		oCPoint* cp = k->pts + j;
		oVec rA = cp->anchorA, rB = cp->anchorB;
		b2r Px = cp->normalImpulse * k->normal.x + cp->tangentImpulse * tX;
		b2r Py = cp->normalImpulse * k->normal.y + cp->tangentImpulse * tY;
		sA.w = sA.w - k->invIA * ( rA.x * Py - rA.y * Px );
		sA.v.x = sA.v.x - k->invMassA * Px;
		sA.v.y = sA.v.y - k->invMassA * Py;
		sB.w = sB.w + k->invIB * ( rB.x * Py - rB.y * Px );
		sB.v.x = sB.v.x + k->invMassB * Px;
		sB.v.y = sB.v.y + k->invMassB * Py;
	}
	store_velocity( w, k->indexA, sA.v, sA.w );
	store_velocity( w, k->indexB, sB.v, sB.w );
}

static void solve_lane( oWorld* w, const oStep* st, oConstraint* k, bool useBias )
{
	oState sA = load_state( w, k->indexA );
	oState sB = load_state( w, k->indexB );
	b2r biasRate = useBias ? k->soft.biasRate : R( 0 );
	b2r massScale = useBias ? k->soft.massScale : R( 1 );
	b2r impulseScale = useBias ? k->soft.impulseScale : R( 0 );
	b2r minBias = -st->pushout;
	oVec dp = ov( sB.dp.x - sA.dp.x, sB.dp.y - sA.dp.y );
	oVec n = k->normal;
	for ( int j = 0; j < 2; ++j )
	{
		oCPoint* cp = k->pts + j;
		oVec rsA = ov( sA.dq.c * cp->anchorA.x - sA.dq.s * cp->anchorA.y, sA.dq.s * cp->anchorA.x + sA.dq.c * cp->anchorA.y );
		oVec rsB = ov( sB.dq.c * cp->anchorB.x - sB.dq.s * cp->anchorB.y, sB.dq.s * cp->anchorB.x + sB.dq.c * cp->anchorB.y );
		oVec ds = ov( dp.x + ( rsB.x - rsA.x ), dp.y + ( rsB.y - rsA.y ) );
		b2r s = ( n.x * ds.x + n.y * ds.y ) + cp->baseSeparation;
		b2r specBias = s * st->inv_h;
		b2r softBias = omax( biasRate * s, minBias );
		b2r bias = s > R( 0 ) ? specBias : softBias;
		oVec rA = cp->anchorA, rB = cp->anchorB;
		b2r dvx = ( sB.v.x - sB.w * rB.y ) - ( sA.v.x - sA.w * rA.y );
		b2r dvy = ( sB.v.y + sB.w * rB.x ) - ( sA.v.y + sA.w * rA.x );
		b2r vn = dvx * n.x + dvy * n.y;
		b2r negImpulse = cp->normalMass * ( massScale * ( vn + bias ) ) + impulseScale * cp->normalImpulse;
		b2r newImpulse = omax( cp->normalImpulse - negImpulse, R( 0 ) );
		b2r impulse = newImpulse - cp->normalImpulse;
		cp->normalImpulse = newImpulse;
		cp->maxNormalImpulse = omax( cp->maxNormalImpulse, newImpulse );
		apply_impulse_lane( &sA.v, &sA.w, &sB.v, &sB.w, k, rA, rB, impulse * n.x, impulse * n.y );
	}
	b2r tX = n.y;
	b2r tY = R( 0 ) - n.x;
	for ( int j = 0; j < 2; ++j )
	{
		oCPoint* cp = k->pts + j;
		oVec rA = cp->anchorA, rB = cp->anchorB;
		b2r dvx = ( sB.v.x - sB.w * rB.y ) - ( sA.v.x - sA.w * rA.y );
		b2r dvy = ( sB.v.y + sB.w * rB.x ) - ( sA.v.y + sA.w * rA.x );
		b2r vt = dvx * tX + dvy * tY;
		b2r negImpulse = cp->tangentMass * vt;
		b2r maxFriction = k->friction * cp->normalImpulse;
		b2r newImpulse = cp->tangentImpulse - negImpulse;
		b2r lo = R( 0 ) - maxFriction;
		b2r mn = newImpulse < maxFriction ? newImpulse : maxFriction;
		newImpulse = lo > mn ? lo : mn;
		b2r impulse = newImpulse - cp->tangentImpulse;
		cp->tangentImpulse = newImpulse;
		apply_impulse_lane( &sA.v, &sA.w, &sB.v, &sB.w, k, rA, rB, impulse * tX, impulse * tY );
	}
	store_velocity( w, k->indexA, sA.v, sA.w );
	store_velocity( w, k->indexB, sB.v, sB.w );
}

static void restitution_lane( oWorld* w, const oStep* st, oConstraint* k )
{
	oState sA = load_state( w, k->indexA );
	oState sB = load_state( w, k->indexB );
	oVec n = k->normal;
	for ( int j = 0; j < 2; ++j )
	{
		oCPoint* cp = k->pts + j;
		bool skip = ( cp->relativeVelocity + st->restitutionThreshold > R( 0 ) ) || ( cp->maxNormalImpulse == R( 0 ) );
		b2r mass = skip ? R( 0 ) : cp->normalMass;
		oVec rA = cp->anchorA, rB = cp->anchorB;
		b2r dvx = ( sB.v.x - sB.w * rB.y ) - ( sA.v.x - sA.w * rA.y );
		b2r dvy = ( sB.v.y + sB.w * rB.x ) - ( sA.v.y + sA.w * rA.x );
		b2r vn = dvx * n.x + dvy * n.y;
		b2r negImpulse = mass * ( vn + k->restitution * cp->relativeVelocity );
		b2r newImpulse = omax( cp->normalImpulse - negImpulse, R( 0 ) );
		b2r impulse = newImpulse - cp->normalImpulse;
		cp->normalImpulse = newImpulse;
		apply_impulse_lane( &sA.v, &sA.w, &sB.v, &sB.w, k, rA, rB, impulse * n.x, impulse * n.y );
	}
	store_velocity( w, k->indexA, sA.v, sA.w );
	store_velocity( w, k->indexB, sB.v, sB.w );
}

/* ------------------------------------------------------------ joints */
static void warm_start_joint( oWorld* w, oJoint* j )
{
	oState sA = load_state( w, j->indexA );
	oState sB = load_state( w, j->indexB );
	o_warm_start_joint( j, &sA, &sB );
	store_velocity( w, j->indexA, sA.v, sA.w );
	store_velocity( w, j->indexB, sB.v, sB.w );
}

static void solve_joint( oWorld* w, const oStep* st, oJoint* j, bool useBias )
{
	oState sA = load_state( w, j->indexA );
	oState sB = load_state( w, j->indexB );
	o_solve_joint( j, st, &sA, &sB, useBias );
	store_velocity( w, j->indexA, sA.v, sA.w );
	store_velocity( w, j->indexB, sB.v, sB.w );
}

/* ------------------------------------------------------------ bodies */
int o_threads = 1;

/* Threads for the oracle's parallel loops (CPU baselines); returns the count in use. */
int b2o_SetThreads( int count )
{
	o_threads = count < 1 ? 1 : count;
	return o_threads;
}

static void integrate_velocities( oWorld* w, const oStep* st )
{
	oVec g = w->gravity;
	b2r h = st->h;
	b2r maxLin = O_MAX_TRANSLATION * st->inv_dt;
	b2r maxAng = O_MAX_ROTATION * st->inv_dt;
	b2r maxLin2 = maxLin * maxLin, maxAng2 = maxAng * maxAng;
	const int n = w->awake.count;
#pragma omp parallel for if ( o_threads > 1 && n >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
	for ( int i = 0; i < n; ++i )
	{
		oBody* b = w->bodies + w->awake.data[i];
		oVec v = b->v;
		b2r a = b->w;
		b2r ld = R( 1 ) / ( R( 1 ) + h * b->linearDamping );
		b2r ad = R( 1 ) / ( R( 1 ) + h * b->angularDamping );
		oVec lvd = omulsv( h * b->invMass, omuladd( b->force, b->mass * b->gravityScale, g ) );
		b2r avd = h * b->invI * b->torque;
		v = omuladd( lvd, ld, v );
		a = avd + ad * a;
		if ( odot( v, v ) > maxLin2 )
		{
			b2r ratio = maxLin / olen( v );
			v = omulsv( ratio, v );
			b->simSpeedCapped = true;
		}
		if ( a * a > maxAng2 )
		{
			b2r ratio = maxAng / oabs( a );
			a *= ratio;
			b->simSpeedCapped = true;
		}
		b->v = v;
		b->w = a;
	}
}

static void integrate_positions( oWorld* w, const oStep* st )
{
	const int n = w->awake.count;
#pragma omp parallel for if ( o_threads > 1 && n >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
	for ( int i = 0; i < n; ++i )
	{
		oBody* b = w->bodies + w->awake.data[i];
		b->dq = ointrot( b->dq, st->h * b->w );
		b->dp = omuladd( b->dp, st->h, b->v );
	}
}

typedef struct oFinalize
{
	uint8_t* enlarged; /* by awake index */
	int* fast;
	int fastCount;
	uint8_t* awakeIslands; /* by awake island index: some body keeps the island awake */
	int splitIslandId;	   /* sleepiest body's island that needs splitting first */
	b2r splitSleepTime;
} oFinalize;

/* reference src/core.h b2_timeToSleep */
#define O_TIME_TO_SLEEP R( 0.5f )

static void finalize_bodies( oWorld* w, const oStep* st, oFinalize* f )
{
	for ( int i = 0; i < w->awake.count; ++i )
	{
		oBody* b = w->bodies + w->awake.data[i];
		oVec v = b->v;
		b2r a = b->w;
		b->center = oadd( b->center, b->dp );
		b->xf.q = onormrot( omulrot( b->dq, b->xf.q ) );
		b2r maxVelocity = olen( v ) + oabs( a ) * b->maxExtent;
		b2r maxDeltaPosition = olen( b->dp ) + oabs( b->dq.s ) * b->maxExtent;
		b2r sleepVelocity = omax( maxVelocity, R( 0.5f ) * st->inv_dt * maxDeltaPosition );
		b->dp = ov( 0, 0 );
		b->dq = orot( 1, 0 );
		b->xf.p = osub( b->center, orotate( b->xf.q, b->localCenter ) );
		b->force = ov( 0, 0 );
		b->torque = 0;
		b->isSpeedCapped = b->simSpeedCapped;
		b->simSpeedCapped = false;
		b->isFast = false;
		if ( w->enableSleep == false || b->enableSleep == false || sleepVelocity > b->sleepThreshold )
		{
			b->sleepTime = 0;
			if ( b->type == b2_dynamicBody && w->enableContinuous && maxVelocity * st->dt > R( 0.5f ) * b->minExtent )
			{
				f->fast[f->fastCount++] = b->id;
				b->isFast = true;
			}
			else
			{
				b->center0 = b->center;
				b->rot0 = b->xf.q;
			}
		}
		else
		{
			b->center0 = b->center;
			b->rot0 = b->xf.q;
			b->sleepTime += st->dt;
		}
		/* any single body keeps its island awake (reference src/solver.c:281-298) */
		oIsland* island = w->islands + b->islandId;
		if ( b->sleepTime < O_TIME_TO_SLEEP )
			f->awakeIslands[island->localIndex] = 1;
		else if ( island->constraintRemoveCount > 0 )
		{
			if ( b->sleepTime > f->splitSleepTime )
			{
				f->splitIslandId = b->islandId;
				f->splitSleepTime = b->sleepTime;
			}
		}
		for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
		{
			oShape* s = w->shapes + sid;
			if ( b->isFast )
			{
				s->isFast = true;
				f->enlarged[i] = 1;
			}
			else
			{
				oBox aabb = o_shape_aabb( s, b->xf );
				aabb.lo.x -= O_SPECULATIVE;
				aabb.lo.y -= O_SPECULATIVE;
				aabb.hi.x += O_SPECULATIVE;
				aabb.hi.y += O_SPECULATIVE;
				s->aabb = aabb;
				if ( obox_contains( s->fatAABB, aabb ) == false )
				{
					s->fatAABB.lo.x = aabb.lo.x - O_AABB_MARGIN;
					s->fatAABB.lo.y = aabb.lo.y - O_AABB_MARGIN;
					s->fatAABB.hi.x = aabb.hi.x + O_AABB_MARGIN;
					s->fatAABB.hi.y = aabb.hi.y + O_AABB_MARGIN;
					s->enlargedAABB = true;
					f->enlarged[i] = 1;
				}
			}
		}
	}
}

static void buffer_move( oWorld* w, int proxyKey )
{
	if ( oset_add( &w->moveSet, (uint64_t)( proxyKey + 1 ) ) == false )
		oia_push( &w->moveArray, proxyKey );
}

/* Continuous collision of a fast body against static shapes (and, for a bullet, against
 * kinematic and dynamic shapes): reference src/solver.c:787-1105.  The query callback
 * filters the candidates and lowers the body's time-of-impact fraction. */
typedef struct oSweepCtx
{
	oWorld* w;
	oShape* fast;
	oBody* fastBody;
	oSweep sweep;
	oVec centroid1, centroid2; /* the fast shape's centroid at the sweep's ends */
	b2r fraction;
} oSweepCtx;

static oSweep body_sweep( const oBody* b )
{
	oSweep s;
	s.c1 = b->center0;
	s.c2 = b->center;
	s.q1 = b->rot0;
	s.q2 = b->xf.q;
	s.localCenter = b->localCenter;
	return s;
}

static bool sweep_query( int proxyId, int shapeId, void* context )
{
	(void)proxyId;
	oSweepCtx* q = (oSweepCtx*)context;
	oWorld* w = q->w;
	if ( shapeId == q->fast->id )
		return true;
	oShape* s = w->shapes + shapeId;
	if ( s->bodyId == q->fast->bodyId )
		return true;
	b2Filter fa = q->fast->filter, fb = s->filter;
	if ( fa.groupIndex == fb.groupIndex && fa.groupIndex != 0 )
	{
		if ( fa.groupIndex <= 0 )
			return true;
	}
	else if ( ( fa.maskBits & fb.categoryBits ) == 0 || ( fa.categoryBits & fb.maskBits ) == 0 )
		return true;
	if ( s->isSensor )
		return true;
	oBody* body = w->bodies + s->bodyId;
	if ( body->isBullet )
		return true;
	if ( o_should_bodies_collide( w, q->fastBody, body ) == false )
		return true;
	/* chain links: skip when the fast shape starts behind or ends in front (reference
	 * src/solver.c:869-885) */
	if ( s->type == b2_smoothSegmentShape )
	{
		oVec p1 = oxfpoint( body->xf, s->smooth.p1 );
		oVec p2 = oxfpoint( body->xf, s->smooth.p2 );
		oVec e = osub( p2, p1 );
		b2r offset1 = ocross( osub( q->centroid1, p1 ), e );
		b2r offset2 = ocross( osub( q->centroid2, p1 ), e );
		if ( offset1 < R( 0 ) || offset2 > R( 0 ) )
			return true;
	}

	oProxy pa = o_shape_proxy( s );
	oProxy pb = o_shape_proxy( q->fast );
	oSweep sa = body_sweep( body );
	int state;
	b2r t = o_time_of_impact( &pa, &sa, &pb, &q->sweep, q->fraction, &state );
	if ( R( 0 ) < t && t < q->fraction )
		q->fraction = t;
	else if ( R( 0 ) == t )
	{
		/* fall back to a small circle around the fast shape's centroid */
		oVec centroid = o_shape_centroid( q->fast );
		pb = o_make_proxy( &centroid, 1, O_SPECULATIVE );
		t = o_time_of_impact( &pa, &sa, &pb, &q->sweep, q->fraction, &state );
		if ( R( 0 ) < t && t < q->fraction )
			q->fraction = t;
	}
	return true;
}

static void solve_continuous( oWorld* w, oBody* b )
{
	oSweepCtx q;
	q.w = w;
	q.fastBody = b;
	q.sweep = body_sweep( b );
	q.fraction = R( 1 );
	oXf xf1, xf2;
	xf1.q = q.sweep.q1;
	xf1.p = osub( q.sweep.c1, orotate( q.sweep.q1, q.sweep.localCenter ) );
	xf2.q = q.sweep.q2;
	xf2.p = osub( q.sweep.c2, orotate( q.sweep.q2, q.sweep.localCenter ) );
	for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
	{
		oShape* s = w->shapes + sid;
		s->isFast = false;
		q.centroid1 = oxfpoint( xf1, s->localCentroid );
		q.centroid2 = oxfpoint( xf2, s->localCentroid );
		oBox box1 = s->aabb;
		oBox box2 = o_shape_aabb( s, xf2 );
		oBox box = obox_union( box1, box2 );
		s->aabb = box2;
		if ( s->isSensor )
			continue;
		q.fast = s;
		otree_query( w->trees + b2_staticBody, box, 0xFFFFFFFFu, sweep_query, &q );
		if ( b->isBullet )
		{
			otree_query( w->trees + b2_kinematicBody, box, 0xFFFFFFFFu, sweep_query, &q );
			otree_query( w->trees + b2_dynamicBody, box, 0xFFFFFFFFu, sweep_query, &q );
		}
	}

	if ( q.fraction < R( 1 ) )
	{
		/* time-of-impact event: move the body back along its sweep */
		oRot rq = onormrot( orot( ( R( 1 ) - q.fraction ) * q.sweep.q1.c + q.fraction * q.sweep.q2.c,
								  ( R( 1 ) - q.fraction ) * q.sweep.q1.s + q.fraction * q.sweep.q2.s ) );
		oVec c = olerp( q.sweep.c1, q.sweep.c2, q.fraction );
		oVec origin = osub( c, orotate( rq, q.sweep.localCenter ) );
		b->xf.p = origin;
		b->xf.q = rq;
		b->center = c;
		b->rot0 = rq;
		b->center0 = c;
		for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
		{
			oShape* s = w->shapes + sid;
			oBox aabb = o_shape_aabb( s, b->xf );
			aabb.lo.x -= O_SPECULATIVE;
			aabb.lo.y -= O_SPECULATIVE;
			aabb.hi.x += O_SPECULATIVE;
			aabb.hi.y += O_SPECULATIVE;
			s->aabb = aabb;
			if ( obox_contains( s->fatAABB, aabb ) == false )
			{
				s->fatAABB.lo.x = aabb.lo.x - O_AABB_MARGIN;
				s->fatAABB.lo.y = aabb.lo.y - O_AABB_MARGIN;
				s->fatAABB.hi.x = aabb.hi.x + O_AABB_MARGIN;
				s->fatAABB.hi.y = aabb.hi.y + O_AABB_MARGIN;
				s->enlargedAABB = true;
				b->enlargeAABB = true;
			}
		}
		w->toiEvents += 1;
		return;
	}

	b->rot0 = b->xf.q;
	b->center0 = b->center;
	for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
	{
		oShape* s = w->shapes + sid;
		if ( obox_contains( s->fatAABB, s->aabb ) == false )
		{
			s->fatAABB.lo.x = s->aabb.lo.x - O_AABB_MARGIN;
			s->fatAABB.lo.y = s->aabb.lo.y - O_AABB_MARGIN;
			s->fatAABB.hi.x = s->aabb.hi.x + O_AABB_MARGIN;
			s->fatAABB.hi.y = s->aabb.hi.y + O_AABB_MARGIN;
			s->enlargedAABB = true;
			b->enlargeAABB = true;
		}
	}
}

/* Continuous collision of one class of fast bodies, then their grown proxies in the
 * dynamic tree (reference src/solver.c:1839-1950: fast bodies first, then bullets, which
 * see the fast bodies' proxies). */
static void continuous_pass( oWorld* w, const int* fast, int count, bool bullets )
{
	for ( int i = 0; i < count; ++i )
		if ( w->bodies[fast[i]].isBullet == bullets )
			solve_continuous( w, w->bodies + fast[i] );
	for ( int i = 0; i < count; ++i )
	{
		oBody* b = w->bodies + fast[i];
		if ( b->isBullet != bullets || b->enlargeAABB == false )
			continue;
		b->enlargeAABB = false;
		for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
		{
			oShape* s = w->shapes + sid;
			if ( s->enlargedAABB == false )
				continue;
			s->enlargedAABB = false;
			otree_enlarge_proxy( w->trees + b2_dynamicBody, s->proxyKey >> 2, s->fatAABB );
		}
	}
}

/* ------------------------------------------------------------ solve */
void o_solve( oWorld* w, b2r dt, int subSteps )
{
	(void)dt;
	oStep st;
	st.subSteps = subSteps < 1 ? 1 : subSteps;
	st.dt = dt;
	st.inv_dt = R( 1 ) / dt;
	st.h = dt / (b2r)st.subSteps;
	st.inv_h = (b2r)st.subSteps * st.inv_dt;
	b2r contactHertz = omin( w->contactHertz, R( 0.25f ) * st.inv_h );
	b2r jointHertz = omin( w->jointHertz, R( 0.125f ) * st.inv_h );
	st.contactSoft = o_make_soft( contactHertz, w->contactDamping, st.h );
	st.staticSoft = o_make_soft( R( 2 ) * contactHertz, w->contactDamping, st.h );
	st.jointSoft = o_make_soft( jointHertz, w->jointDamping, st.h );
	st.restitutionThreshold = w->restitutionThreshold;
	st.pushout = w->pushout;
	st.enableWarmStarting = w->enableWarmStarting;

	w->stepIndex += 1;
	w->inv_h = st.inv_h;
	o_merge_awake_islands( w );
	int awakeCount = w->awake.count;
	if ( awakeCount == 0 )
		return;

	/* active colours 0..10 in order, then the overflow colour */
	int active[O_COLORS];
	int activeCount = 0;
	for ( int i = 0; i < O_OVERFLOW; ++i )
		if ( w->colors[i].contacts.count + w->colors[i].joints.count > 0 )
			active[activeCount++] = i;

	o_capture_inputs( w );
	int totalContacts = 0;
	for ( int i = 0; i < O_COLORS; ++i )
		totalContacts += w->colors[i].contacts.count;
	oConstraint* cons = (oConstraint*)malloc( sizeof( oConstraint ) * (size_t)( totalContacts + 1 ) );
	int colorStart[O_COLORS + 1];
	{
		int n = 0;
		for ( int i = 0; i < O_COLORS; ++i )
		{
			colorStart[i] = n;
			oIntArray* a = &w->colors[i].contacts;
			const int count = a->count;
			oConstraint* base = cons + n;
#pragma omp parallel for if ( o_threads > 1 && count >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
			for ( int k = 0; k < count; ++k )
				prepare_contact( w, &st, base + k, w->contacts + a->data[k] );
			n += count;
		}
		colorStart[O_COLORS] = n;
	}
	for ( int c = 0; c < O_COLORS; ++c )
	{
		oIntArray* j = &w->colors[c].joints;
		for ( int k = 0; k < j->count; ++k )
			o_prepare_joint( w, &st, w->joints + j->data[k] );
	}

	oColor* overflow = w->colors + O_OVERFLOW;
	oConstraint* ocons = cons + colorStart[O_OVERFLOW];
	int ocount = overflow->contacts.count;

	for ( int sub = 0; sub < st.subSteps; ++sub )
	{
		integrate_velocities( w, &st );

		for ( int k = 0; k < overflow->joints.count; ++k )
			warm_start_joint( w, w->joints + overflow->joints.data[k] );
		for ( int k = 0; k < ocount; ++k )
			warm_start_overflow( w, ocons + k );
		if ( st.enableWarmStarting )
		{
			for ( int a = 0; a < activeCount; ++a )
			{
				int c = active[a];
				for ( int k = 0; k < w->colors[c].joints.count; ++k )
					warm_start_joint( w, w->joints + w->colors[c].joints.data[k] );
				const int k0 = colorStart[c], k1 = colorStart[c + 1];
#pragma omp parallel for if ( o_threads > 1 && k1 - k0 >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
				for ( int k = k0; k < k1; ++k )
					warm_start_lane( w, cons + k );
			}
		}

		for ( int k = 0; k < overflow->joints.count; ++k )
			solve_joint( w, &st, w->joints + overflow->joints.data[k], true );
		for ( int k = 0; k < ocount; ++k )
			solve_overflow( w, &st, ocons + k, true );
		for ( int a = 0; a < activeCount; ++a )
		{
			int c = active[a];
			for ( int k = 0; k < w->colors[c].joints.count; ++k )
				solve_joint( w, &st, w->joints + w->colors[c].joints.data[k], true );
			const int k0 = colorStart[c], k1 = colorStart[c + 1];
#pragma omp parallel for if ( o_threads > 1 && k1 - k0 >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
			for ( int k = k0; k < k1; ++k )
				solve_lane( w, &st, cons + k, true );
		}

		integrate_positions( w, &st );

		for ( int k = 0; k < overflow->joints.count; ++k )
			solve_joint( w, &st, w->joints + overflow->joints.data[k], false );
		for ( int k = 0; k < ocount; ++k )
			solve_overflow( w, &st, ocons + k, false );
		for ( int a = 0; a < activeCount; ++a )
		{
			int c = active[a];
			for ( int k = 0; k < w->colors[c].joints.count; ++k )
				solve_joint( w, &st, w->joints + w->colors[c].joints.data[k], false );
			const int k0 = colorStart[c], k1 = colorStart[c + 1];
#pragma omp parallel for if ( o_threads > 1 && k1 - k0 >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
			for ( int k = k0; k < k1; ++k )
				solve_lane( w, &st, cons + k, false );
		}
	}

	for ( int k = 0; k < ocount; ++k )
		restitution_overflow( w, &st, ocons + k );
	for ( int a = 0; a < activeCount; ++a )
	{
		int c = active[a];
		const int k0 = colorStart[c], k1 = colorStart[c + 1];
#pragma omp parallel for if ( o_threads > 1 && k1 - k0 >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
		for ( int k = k0; k < k1; ++k )
			restitution_lane( w, &st, cons + k );
	}

	/* store impulses: the overflow path writes existing points, the 8-lane path both */
	const int stored = colorStart[O_COLORS];
#pragma omp parallel for if ( o_threads > 1 && stored >= O_PARALLEL_MIN ) num_threads( o_threads ) schedule( static )
	for ( int k = 0; k < stored; ++k )
	{
		oConstraint* c = cons + k;
		oManifold* m = &w->contacts[c->contactId].manifold;
		bool lane = k < colorStart[O_OVERFLOW];
		int n = lane ? 2 : m->count;
		for ( int j = 0; j < n; ++j )
		{
			m->pts[j].normalImpulse = c->pts[j].normalImpulse;
			m->pts[j].tangentImpulse = c->pts[j].tangentImpulse;
			m->pts[j].maxNormalImpulse = c->pts[j].maxNormalImpulse;
			m->pts[j].normalVelocity = c->pts[j].relativeVelocity;
		}
	}
	free( cons );
	o_capture_outputs( w );
	o_report_hits( w );

	/* the previous step's split candidate is split beside the constraint solver, before
	 * the bodies are finalised (reference src/solver.c:1395-1410, :1614-1620) */
	if ( w->splitIslandId != O_NULL )
		o_split_island( w, w->splitIslandId );
	w->splitIslandId = O_NULL;

	oFinalize f;
	f.enlarged = (uint8_t*)calloc( (size_t)awakeCount, 1 );
	f.fast = (int*)malloc( sizeof( int ) * (size_t)awakeCount );
	f.fastCount = 0;
	f.awakeIslands = (uint8_t*)calloc( (size_t)( w->awakeIslands.count > 0 ? w->awakeIslands.count : 1 ), 1 );
	f.splitIslandId = O_NULL;
	f.splitSleepTime = 0;
	finalize_bodies( w, &st, &f );

	/* enlarge proxies in awake order (reference src/solver.c:1741-1797) */
	for ( int i = 0; i < awakeCount; ++i )
	{
		if ( f.enlarged[i] == 0 )
			continue;
		oBody* b = w->bodies + w->awake.data[i];
		for ( int sid = b->headShape; sid != O_NULL; sid = w->shapes[sid].next )
		{
			oShape* s = w->shapes + sid;
			if ( s->enlargedAABB )
			{
				otree_enlarge_proxy( w->trees + ( s->proxyKey & 3 ), s->proxyKey >> 2, s->fatAABB );
				buffer_move( w, s->proxyKey );
				s->enlargedAABB = false;
			}
			else if ( s->isFast )
			{
				buffer_move( w, s->proxyKey );
			}
		}
	}

	continuous_pass( w, f.fast, f.fastCount, false );
	continuous_pass( w, f.fast, f.fastCount, true );

	/* island sleep, last because it moves bodies out of the awake set (reference
	 * src/solver.c:1956-2001): keep the split candidate for the next step, then try the
	 * islands no body kept awake, in reverse so that removal keeps the rest in place */
	if ( w->enableSleep )
	{
		if ( f.splitIslandId != O_NULL && f.splitSleepTime > R( 0 ) )
			w->splitIslandId = f.splitIslandId;
		for ( int i = w->awakeIslands.count - 1; i >= 0; --i )
		{
			if ( f.awakeIslands[i] )
				continue;
			o_try_sleep_island( w, w->awakeIslands.data[i] );
		}
	}
	free( f.awakeIslands );
	free( f.enlarged );
	free( f.fast );
}

void o_step( oWorld* w, b2r dt, int subSteps )
{
	o_update_pairs( w );
	o_collide( w );
	if ( dt > R( 0 ) )
		o_solve( w, dt, subSteps );
}

/* ------------------------------------------------------------ solver-stage capture */
/* Test hook: records the inputs of the solver stage (after the narrowphase and the
 * colouring) and its outputs (after impulses are stored, before bodies are finalised),
 * in the layouts of b2ContactSolveDesc (include/box2d/gpu.h). */
typedef struct b2oCapture
{
	int bodyCap, contactCap;
	int bodyCount, awakeCount, contactCount, overflow;
	float *statesIn, *statesOut, *mass, *force, *damping;
	int* awake;
	int* contactBodies;
	float* mix;
	b2Manifold *manifoldsIn, *manifoldsOut;
	int colorStart[13];
} b2oCapture;

static b2oCapture* s_capture;

static void capture_states( oWorld* w, float* out )
{
	for ( int i = 0; i < w->bodyIds.next; ++i )
	{
		oBody* b = w->bodies + i;
		float* o = out + 8 * i;
		bool moving = b->id == i && b->type != b2_staticBody;
		o[0] = moving ? (float)b->v.x : 0.0f;
		o[1] = moving ? (float)b->v.y : 0.0f;
		o[2] = moving ? (float)b->w : 0.0f;
		o[3] = 0.0f;
		o[4] = moving ? (float)b->dp.x : 0.0f;
		o[5] = moving ? (float)b->dp.y : 0.0f;
		o[6] = moving ? (float)b->dq.c : 1.0f;
		o[7] = moving ? (float)b->dq.s : 0.0f;
	}
}

static void capture_manifolds( oWorld* w, b2Manifold* out )
{
	int n = 0;
	for ( int c = 0; c < O_COLORS; ++c )
	{
		oIntArray* a = &w->colors[c].contacts;
		for ( int k = 0; k < a->count; ++k )
		{
			const oManifold* m = &w->contacts[a->data[k]].manifold;
			b2Manifold* o = out + n++;
			memset( o, 0, sizeof( *o ) );
			o->normal.x = (float)m->normal.x;
			o->normal.y = (float)m->normal.y;
			o->pointCount = m->count;
			for ( int j = 0; j < 2; ++j )
			{
				const oMPoint* p = m->pts + j;
				b2ManifoldPoint* q = o->points + j;
				q->point = vfo( p->point );
				q->anchorA = vfo( p->anchorA );
				q->anchorB = vfo( p->anchorB );
				q->separation = (float)p->separation;
				q->normalImpulse = (float)p->normalImpulse;
				q->tangentImpulse = (float)p->tangentImpulse;
				q->maxNormalImpulse = (float)p->maxNormalImpulse;
				q->normalVelocity = (float)p->normalVelocity;
				q->id = p->id;
				q->persisted = p->persisted;
			}
		}
	}
}

void o_capture_inputs( oWorld* w )
{
	b2oCapture* cap = s_capture;
	if ( cap == NULL )
		return;
	int nb = w->bodyIds.next;
	int nc = 0;
	for ( int c = 0; c < O_COLORS; ++c )
		nc += w->colors[c].contacts.count;
	cap->bodyCount = nb;
	cap->awakeCount = w->awake.count;
	cap->contactCount = nc;
	if ( nb > cap->bodyCap || nc > cap->contactCap || w->awake.count > cap->bodyCap )
	{
		cap->overflow = 1;
		return;
	}
	capture_states( w, cap->statesIn );
	for ( int i = 0; i < nb; ++i )
	{
		oBody* b = w->bodies + i;
		float* m = cap->mass + 4 * i;
		float* f = cap->force + 4 * i;
		float* d = cap->damping + 4 * i;
		m[0] = (float)b->mass;
		m[1] = (float)b->invMass;
		m[2] = (float)b->inertia;
		m[3] = (float)b->invI;
		f[0] = (float)b->force.x;
		f[1] = (float)b->force.y;
		f[2] = (float)b->torque;
		f[3] = (float)b->gravityScale;
		d[0] = (float)b->linearDamping;
		d[1] = (float)b->angularDamping;
		d[2] = (float)b->minExtent;
		d[3] = (float)b->maxExtent;
	}
	memcpy( cap->awake, w->awake.data, sizeof( int ) * (size_t)w->awake.count );
	int n = 0;
	for ( int c = 0; c < O_COLORS; ++c )
	{
		cap->colorStart[c] = n;
		oIntArray* a = &w->colors[c].contacts;
		for ( int k = 0; k < a->count; ++k )
		{
			oContact* ct = w->contacts + a->data[k];
			cap->contactBodies[2 * n] = ct->simIndexA;
			cap->contactBodies[2 * n + 1] = ct->simIndexB;
			cap->mix[2 * n] = (float)ct->friction;
			cap->mix[2 * n + 1] = (float)ct->restitution;
			n += 1;
		}
	}
	cap->colorStart[O_COLORS] = n;
	capture_manifolds( w, cap->manifoldsIn );
}

void o_capture_outputs( oWorld* w )
{
	b2oCapture* cap = s_capture;
	if ( cap == NULL || cap->overflow )
		return;
	capture_states( w, cap->statesOut );
	capture_manifolds( w, cap->manifoldsOut );
}

/* Steps the world once, capturing the solver stage's inputs and outputs. */
int b2o_StepCapture( b2WorldId worldId, float timeStep, int subStepCount, b2oCapture* cap )
{
	cap->overflow = 0;
	s_capture = cap;
	b2World_Step( worldId, timeStep, subStepCount );
	s_capture = NULL;
	return cap->overflow ? -1 : 0;
}
