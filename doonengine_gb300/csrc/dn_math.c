/*
 * dn_math.c -- vector / matrix helpers of the DN_* API (see dn_math.h).
 *
 * Restated from the underlying maths, not from the reference's vendored
 * header: Tait-Bryan Z*Y*X rotation, the OpenGL-style perspective frustum,
 * a right-handed look-at basis, and a cofactor (adjugate / determinant)
 * inverse.  Compiled with -ffp-contract=off so results do not depend on FMA
 * contraction.  Matrices are column-major, m[col][row].
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
	/* Laplace expansion by 2x2 minors of columns (0,1) and (2,3):
	 * det = sum of products of complementary minors; inverse = adjugate / det */
	float a[4][4];
	memcpy(a, in.m, sizeof(a));   /* a[col][row] */
	/* element (row r, col c) = a[c][r] */
#define E(r, c) a[c][r]
	float s0 = E(0,0) * E(1,1) - E(1,0) * E(0,1);
	float s1 = E(0,0) * E(1,2) - E(1,0) * E(0,2);
	float s2 = E(0,0) * E(1,3) - E(1,0) * E(0,3);
	float s3 = E(0,1) * E(1,2) - E(1,1) * E(0,2);
	float s4 = E(0,1) * E(1,3) - E(1,1) * E(0,3);
	float s5 = E(0,2) * E(1,3) - E(1,2) * E(0,3);
	float c5 = E(2,2) * E(3,3) - E(3,2) * E(2,3);
	float c4 = E(2,1) * E(3,3) - E(3,1) * E(2,3);
	float c3 = E(2,1) * E(3,2) - E(3,1) * E(2,2);
	float c2 = E(2,0) * E(3,3) - E(3,0) * E(2,3);
	float c1 = E(2,0) * E(3,2) - E(3,0) * E(2,2);
	float c0 = E(2,0) * E(3,1) - E(3,0) * E(2,1);
	float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
	DNmat4 r;
	memset(&r, 0, sizeof(r));
	if (det == 0.0f) return r;
	float id = 1.0f / det;
	float b[4][4];   /* b[row][col] of the inverse */
	b[0][0] = ( E(1,1) * c5 - E(1,2) * c4 + E(1,3) * c3) * id;
	b[0][1] = (-E(0,1) * c5 + E(0,2) * c4 - E(0,3) * c3) * id;
	b[0][2] = ( E(3,1) * s5 - E(3,2) * s4 + E(3,3) * s3) * id;
	b[0][3] = (-E(2,1) * s5 + E(2,2) * s4 - E(2,3) * s3) * id;
	b[1][0] = (-E(1,0) * c5 + E(1,2) * c2 - E(1,3) * c1) * id;
	b[1][1] = ( E(0,0) * c5 - E(0,2) * c2 + E(0,3) * c1) * id;
	b[1][2] = (-E(3,0) * s5 + E(3,2) * s2 - E(3,3) * s1) * id;
	b[1][3] = ( E(2,0) * s5 - E(2,2) * s2 + E(2,3) * s1) * id;
	b[2][0] = ( E(1,0) * c4 - E(1,1) * c2 + E(1,3) * c0) * id;
	b[2][1] = (-E(0,0) * c4 + E(0,1) * c2 - E(0,3) * c0) * id;
	b[2][2] = ( E(3,0) * s4 - E(3,1) * s2 + E(3,3) * s0) * id;
	b[2][3] = (-E(2,0) * s4 + E(2,1) * s2 - E(2,3) * s0) * id;
	b[3][0] = (-E(1,0) * c3 + E(1,1) * c1 - E(1,2) * c0) * id;
	b[3][1] = ( E(0,0) * c3 - E(0,1) * c1 + E(0,2) * c0) * id;
	b[3][2] = (-E(3,0) * s3 + E(3,1) * s1 - E(3,2) * s0) * id;
	b[3][3] = ( E(2,0) * s3 - E(2,1) * s1 + E(2,2) * s0) * id;
#undef E
	for (int row = 0; row < 4; row++)
		for (int col = 0; col < 4; col++) r.m[col][row] = b[row][col];
	return r;
}
