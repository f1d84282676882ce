/*
 * dn_math.c -- vector / matrix helpers of the DN_* API (see dn_math.h).
 *
 * Tait-Bryan Z*Y*X rotation, the OpenGL-style perspective frustum and a
 * right-handed look-at basis are restated from the underlying maths.  The
 * cofactor (adjugate / determinant) inverse DN_mat4_inv and the quaternion
 * helpers follow the reference's vendored math header (QuickMath,
 * quickmath.h mat4_inv and the quaternion functions) operation by operation,
 * because the camera matrices and shape transforms must be bit-identical to
 * the reference's.  Compiled with -ffp-contract=off so results do not depend
 * on FMA contraction.  Matrices are column-major, m[col][row].
 */
#include "DoonEngine/dn_math.h"
#include <math.h>
#include <string.h>

float DN_deg_to_rad(float deg) { return deg * 0.01745329251f; }

DNvec3 DN_vec3_add(DNvec3 a, DNvec3 b) { DNvec3 r = {{a.x + b.x, a.y + b.y, a.z + b.z}}; return r; }
DNvec3 DN_vec3_sub(DNvec3 a, DNvec3 b) { DNvec3 r = {{a.x - b.x, a.y - b.y, a.z - b.z}}; return r; }
DNvec3 DN_vec3_scale(DNvec3 v, float s) { DNvec3 r = {{v.x * s, v.y * s, v.z * s}}; return r; }
float DN_vec3_dot(DNvec3 a, DNvec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

DNvec3 DN_vec3_cross(DNvec3 a, DNvec3 b)
{
	DNvec3 r = {{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}};
	return r;
}

float DN_vec3_length(DNvec3 v) { return sqrtf(DN_vec3_dot(v, v)); }

DNvec3 DN_vec3_normalize(DNvec3 v)
{
	DNvec3 r = {{0.0f, 0.0f, 0.0f}};
	float len = DN_vec3_length(v);
	if (len != 0.0f) {
		float inv = 1.0f / len;
		r.x = v.x * inv; r.y = v.y * inv; r.z = v.z * inv;
	}
	return r;
}

DNvec3 DN_mat3_mult_vec3(DNmat3 m, DNvec3 v)
{
	DNvec3 r;
	for (int row = 0; row < 3; row++)
		r.v[row] = m.m[0][row] * v.x + m.m[1][row] * v.y + m.m[2][row] * v.z;
	return r;
}

DNmat4 DN_mat4_identity(void)
{
	DNmat4 r;
	memset(&r, 0, sizeof(r));
	r.m[0][0] = r.m[1][1] = r.m[2][2] = r.m[3][3] = 1.0f;
	return r;
}

DNmat4 DN_mat4_mult(DNmat4 a, DNmat4 b)
{
	/* (a*b)[col][row] = sum_k a[k][row] * b[col][k], k ascending */
	DNmat4 r;
	for (int col = 0; col < 4; col++)
		for (int row = 0; row < 4; row++)
			r.m[col][row] = a.m[0][row] * b.m[col][0] + a.m[1][row] * b.m[col][1] +
			                a.m[2][row] * b.m[col][2] + a.m[3][row] * b.m[col][3];
	return r;
}

DNvec4 DN_mat4_mult_vec4(DNmat4 m, DNvec4 v)
{
	DNvec4 r;
	for (int row = 0; row < 4; row++)
		r.v[row] = m.m[0][row] * v.x + m.m[1][row] * v.y + m.m[2][row] * v.z + m.m[3][row] * v.w;
	return r;
}

DNmat4 DN_mat4_rotate_euler(DNvec3 a)
{
	/* R = Rz(roll) * Ry(yaw) * Rx(pitch) */
	float x = DN_deg_to_rad(a.x), y = DN_deg_to_rad(a.y), z = DN_deg_to_rad(a.z);
	float sx = sinf(x), cx = cosf(x), sy = sinf(y), cy = cosf(y), sz = sinf(z), cz = cosf(z);
	DNmat4 r = DN_mat4_identity();
	r.m[0][0] = cy * cz;
	r.m[0][1] = cy * sz;
	r.m[0][2] = -sy;
	r.m[1][0] = sx * sy * cz - cx * sz;
	r.m[1][1] = sx * sy * sz + cx * cz;
	r.m[1][2] = sx * cy;
	r.m[2][0] = cx * sy * cz + sx * sz;
	r.m[2][1] = cx * sy * sz - sx * cz;
	r.m[2][2] = cx * cy;
	return r;
}

DNmat3 DN_mat4_top_left(DNmat4 m)
{
	DNmat3 r;
	for (int c = 0; c < 3; c++)
		for (int k = 0; k < 3; k++) r.m[c][k] = m.m[c][k];
	return r;
}

DNmat4 DN_mat4_perspective(float fov, float aspect, float n, float f)
{
	/* symmetric frustum with half-height tan(fov/2)*near */
	DNmat4 r;
	memset(&r, 0, sizeof(r));
	float top = tanf(DN_deg_to_rad(fov * 0.5f)) * n;
	float right = aspect * top;
	r.m[0][0] = n / right;
	r.m[1][1] = n / top;
	r.m[2][2] = -(f + n) / (f - n);
	r.m[3][2] = -2.0f * f * n / (f - n);
	r.m[2][3] = -1.0f;
	return r;
}

DNmat4 DN_mat4_lookat(DNvec3 pos, DNvec3 target, DNvec3 up)
{
	/* basis rows (right, up, back) followed by the translation by -pos */
	DNvec3 back = DN_vec3_normalize(DN_vec3_sub(pos, target));
	DNvec3 right = DN_vec3_normalize(DN_vec3_cross(up, back));
	DNvec3 u = DN_vec3_cross(back, right);
	DNmat4 basis = DN_mat4_identity();
	basis.m[0][0] = right.x; basis.m[1][0] = right.y; basis.m[2][0] = right.z;
	basis.m[0][1] = u.x;     basis.m[1][1] = u.y;     basis.m[2][1] = u.z;
	basis.m[0][2] = back.x;  basis.m[1][2] = back.y;  basis.m[2][2] = back.z;
	DNmat4 t = DN_mat4_identity();
	t.m[3][0] = -pos.x; t.m[3][1] = -pos.y; t.m[3][2] = -pos.z;
	return DN_mat4_mult(basis, t);
}

DNmat4 DN_mat4_inv(DNmat4 in)
{
	/* Adjugate / determinant.  The cofactors come from six 2x2 minors of two columns at a time, and the
	 * operations run in the order of the reference's math header (quickmath.h mat4_inv), so the inverse is
	 * bit-identical to the reference's, signed zeros included.  A singular matrix returns all zeros. */
	const float a = in.m[0][0], b = in.m[0][1], c = in.m[0][2], d = in.m[0][3];
	const float e = in.m[1][0], f = in.m[1][1], g = in.m[1][2], h = in.m[1][3];
	const float i = in.m[2][0], j = in.m[2][1], k = in.m[2][2], l = in.m[2][3];
	const float m = in.m[3][0], n = in.m[3][1], o = in.m[3][2], p = in.m[3][3];
	DNmat4 r;
	float t0, t1, t2, t3, t4, t5;

	/* minors of columns 2 and 3 */
	t0 = k * p - o * l; t1 = j * p - n * l; t2 = j * o - n * k;
	t3 = i * p - m * l; t4 = i * o - m * k; t5 = i * n - m * j;
	r.m[0][0] =   f * t0 - g * t1 + h * t2;
	r.m[1][0] = -(e * t0 - g * t3 + h * t4);
	r.m[2][0] =   e * t1 - f * t3 + h * t5;
	r.m[3][0] = -(e * t2 - f * t4 + g * t5);
	r.m[0][1] = -(b * t0 - c * t1 + d * t2);
	r.m[1][1] =   a * t0 - c * t3 + d * t4;
	r.m[2][1] = -(a * t1 - b * t3 + d * t5);
	r.m[3][1] =   a * t2 - b * t4 + c * t5;

	/* minors of columns 1 and 3 */
	t0 = g * p - o * h; t1 = f * p - n * h; t2 = f * o - n * g;
	t3 = e * p - m * h; t4 = e * o - m * g; t5 = e * n - m * f;
	r.m[0][2] =   b * t0 - c * t1 + d * t2;
	r.m[1][2] = -(a * t0 - c * t3 + d * t4);
	r.m[2][2] =   a * t1 - b * t3 + d * t5;
	r.m[3][2] = -(a * t2 - b * t4 + c * t5);

	/* minors of columns 1 and 2 */
	t0 = g * l - k * h; t1 = f * l - j * h; t2 = f * k - j * g;
	t3 = e * l - i * h; t4 = e * k - i * g; t5 = e * j - i * f;
	r.m[0][3] = -(b * t0 - c * t1 + d * t2);
	r.m[1][3] =   a * t0 - c * t3 + d * t4;
	r.m[2][3] = -(a * t1 - b * t3 + d * t5);
	r.m[3][3] =   a * t2 - b * t4 + c * t5;

	const float det = a * r.m[0][0] + b * r.m[1][0] + c * r.m[2][0] + d * r.m[3][0];
	if (det == 0.0f) {
		memset(&r, 0, sizeof(r));
		return r;
	}
	const float s = 1.0f / det;
	for (int col = 0; col < 4; col++)
		for (int row = 0; row < 4; row++) r.m[col][row] = r.m[col][row] * s;
	return r;
}

DNmat4 DN_mat4_translate(DNvec3 t)
{
	DNmat4 r = DN_mat4_identity();
	r.m[3][0] = t.x; r.m[3][1] = t.y; r.m[3][2] = t.z;
	return r;
}

DNquaternion DN_quaternion_identity(void)
{
	DNquaternion q = {{0.0f, 0.0f, 0.0f, 1.0f}};
	return q;
}

DNquaternion DN_quaternion_from_euler(DNvec3 a)
{
	/* half angles; q = qx * qy * qz expanded (the reference's shape examples build orientations this
	 * way, main.c:107-108), each product evaluated as (x-term * y-term) * z-term */
	const float hx = DN_deg_to_rad(a.x * 0.5f), hy = DN_deg_to_rad(a.y * 0.5f), hz = DN_deg_to_rad(a.z * 0.5f);
	const float sx = sinf(hx), cx = cosf(hx), sy = sinf(hy), cy = cosf(hy), sz = sinf(hz), cz = cosf(hz);
	DNquaternion q;
	q.x = sx * cy * cz - cx * sy * sz;
	q.y = cx * sy * cz + sx * cy * sz;
	q.z = cx * cy * sz - sx * sy * cz;
	q.w = cx * cy * cz + sx * sy * sz;
	return q;
}

DNmat4 DN_quaternion_to_mat4(DNquaternion q)
{
	/* rotation matrix of a unit quaternion from the doubled products (x2 = 2x etc.), stored so that
	 * m[0][1] = 2(xy - wz): the transpose of the matrix that rotates column vectors by q, which is the
	 * layout the reference's shape transforms are built from (voxelShapes.c:323-324) */
	const float x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
	const float xx = q.x * x2, xy = q.x * y2, xz = q.x * z2;
	const float yy = q.y * y2, yz = q.y * z2, zz = q.z * z2;
	const float wx = q.w * x2, wy = q.w * y2, wz = q.w * z2;
	DNmat4 r = DN_mat4_identity();
	r.m[0][0] = 1.0f - (yy + zz); r.m[0][1] = xy - wz;          r.m[0][2] = xz + wy;
	r.m[1][0] = xy + wz;          r.m[1][1] = 1.0f - (xx + zz); r.m[1][2] = yz - wx;
	r.m[2][0] = xz - wy;          r.m[2][1] = yz + wx;          r.m[2][2] = 1.0f - (xx + yy);
	return r;
}
