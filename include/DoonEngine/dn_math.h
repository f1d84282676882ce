/*
 * dn_math.h -- the vector / matrix types of the DoonEngine API and the camera
 * math the draw path needs.
 *
 * The reference takes these types from a vendored third-party header
 * (dependencies/include/QuickMath/quickmath.h, typedefs at 185-190) that
 * forces SSE and does not build on Arm.  This header keeps the same names and
 * memory layouts (3 floats per DNvec3; column-major DNmat4, m[col][row]) and
 * restates, from the underlying maths, only the functions the API uses.
 */
#ifndef DN_MATH_H
#define DN_MATH_H

#ifdef __cplusplus
extern "C" {
#endif

typedef union DNvec2 { float v[2]; struct { float x, y; }; } DNvec2;
typedef union DNvec3 { float v[3]; struct { float x, y, z; }; struct { float r, g, b; }; } DNvec3;
typedef union DNvec4 { float v[4]; struct { float x, y, z, w; }; } DNvec4;
typedef union DNmat3 { float m[3][3]; } DNmat3;     /* column-major m[col][row] */
typedef union DNmat4 { float m[4][4]; } DNmat4;     /* column-major m[col][row] */
typedef union DNquaternion { float q[4]; struct { float x, y, z, w; }; } DNquaternion;   /* w the real part */

float DN_deg_to_rad(float deg);
DNvec3 DN_vec3_add(DNvec3 a, DNvec3 b);
DNvec3 DN_vec3_sub(DNvec3 a, DNvec3 b);
DNvec3 DN_vec3_scale(DNvec3 v, float s);
float DN_vec3_dot(DNvec3 a, DNvec3 b);
DNvec3 DN_vec3_cross(DNvec3 a, DNvec3 b);
float DN_vec3_length(DNvec3 v);
/* v * (1 / |v|); the zero vector stays zero */
DNvec3 DN_vec3_normalize(DNvec3 v);
DNvec3 DN_mat3_mult_vec3(DNmat3 m, DNvec3 v);
DNmat4 DN_mat4_identity(void);
DNmat4 DN_mat4_mult(DNmat4 a, DNmat4 b);
DNvec4 DN_mat4_mult_vec4(DNmat4 m, DNvec4 v);
/* rotation from Euler angles in degrees {pitch (x), yaw (y), roll (z)}: R = Rz * Ry * Rx applied to column vectors */
DNmat4 DN_mat4_rotate_euler(DNvec3 anglesDeg);
DNmat3 DN_mat4_top_left(DNmat4 m);
/* right-handed perspective; aspect = width / height of the frustum */
DNmat4 DN_mat4_perspective(float fovDeg, float aspect, float nearPlane, float farPlane);
/* view matrix looking from pos towards target */
DNmat4 DN_mat4_lookat(DNvec3 pos, DNvec3 target, DNvec3 up);
/* general 4x4 inverse by cofactor expansion; a singular matrix returns all zeros */
DNmat4 DN_mat4_inv(DNmat4 m);
/* translation by t */
DNmat4 DN_mat4_translate(DNvec3 t);
DNquaternion DN_quaternion_identity(void);
/* rotation from Euler angles in degrees {x, y, z}: the product of the three half-angle rotations about x,
 * y and z, written out component by component */
DNquaternion DN_quaternion_from_euler(DNvec3 anglesDeg);
/* rotation matrix of a unit quaternion, m[0][1] = 2(xy - wz) (the layout the shape functions use) */
DNmat4 DN_quaternion_to_mat4(DNquaternion q);

#ifdef __cplusplus
}
#endif

#endif
