// view.cpp — host-side cull-uniform builder (blz_view_setup).
//
// Produces the same CameraViewData bytes as the reference camera: SetupCamera + UpdateProjection
// (src/Game/blitzenCamera.cpp:14-41,93-126) over the BlitML helpers they call
// (src/BlitzenMathLibrary/blitML.h:261-278 InfiniteZPerspective, 312-363 Mat4Inverse,
// 497-534 NormalizeQuat/QuatToMat4, 559-570 QuatFromAngleAxis; blitMLTypes.h:150-193 Transpose
// and the matrix products). Every product and sum is kept in the reference's order so the result
// is bit-identical; this file is compiled with -ffp-contract=off for that reason.
#include <array>
#include <cmath>
#include <cstring>

#include "../../include/blz_cull.h"

namespace {

using Mat = std::array<float, 16>;  // column-major: (row r, column c) at [c * 4 + r]

Mat identity() {
    Mat m{};
    m[0] = m[5] = m[10] = m[15] = 1.0f;
    return m;
}

// (a * b)[j + 4i] = a[j]*b[4i] + a[4+j]*b[4i+1] + a[8+j]*b[4i+2] + a[12+j]*b[4i+3]
Mat multiply(const Mat& a, const Mat& b) {
    Mat r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float acc = a[j] * b[4 * i];
            acc = acc + a[4 + j] * b[4 * i + 1];
            acc = acc + a[8 + j] * b[4 * i + 2];
            acc = acc + a[12 + j] * b[4 * i + 3];
            r[j + 4 * i] = acc;
        }
    return r;
}

// Rotation matrix of a quaternion after normalising it.
Mat rotation(float qx, float qy, float qz, float qw) {
    const float len = std::sqrt(qx * qx + qy * qy + qz * qz + qw * qw);
    const float x = qx / len, y = qy / len, z = qz / len, w = qw / len;
    Mat m = identity();
    m[0] = 1.0f - 2.0f * y * y - 2.0f * z * z;
    m[1] = 2.0f * x * y - 2.0f * z * w;
    m[2] = 2.0f * x * z + 2.0f * y * w;
    m[4] = 2.0f * x * y + 2.0f * z * w;
    m[5] = 1.0f - 2.0f * x * x - 2.0f * z * z;
    m[6] = 2.0f * y * z - 2.0f * x * w;
    m[8] = 2.0f * x * z - 2.0f * y * w;
    m[9] = 2.0f * y * z + 2.0f * x * w;
    m[10] = 1.0f - 2.0f * x * x - 2.0f * y * y;
    return m;
}

// Inverse by 2x2 sub-determinant products (the cofactor scheme of the reference's Mat4Inverse,
// with its exact grouping of products and sums).
Mat inverse(const Mat& m) {
    // pairwise products of the lower two rows' entries (columns 2/3 then 0/1 blocks)
    const float a0 = m[10] * m[15], a1 = m[14] * m[11], a2 = m[6] * m[15], a3 = m[14] * m[7];
    const float a4 = m[6] * m[11], a5 = m[10] * m[7], a6 = m[2] * m[15], a7 = m[14] * m[3];
    const float a8 = m[2] * m[11], a9 = m[10] * m[3], a10 = m[2] * m[7], a11 = m[6] * m[3];
    const float b0 = m[8] * m[13], b1 = m[12] * m[9], b2 = m[4] * m[13], b3 = m[12] * m[5];
    const float b4 = m[4] * m[9], b5 = m[8] * m[5], b6 = m[0] * m[13], b7 = m[12] * m[1];
    const float b8 = m[0] * m[9], b9 = m[8] * m[1], b10 = m[0] * m[5], b11 = m[4] * m[1];
    Mat o{};
    o[0] = (a0 * m[5] + a3 * m[9] + a4 * m[13]) - (a1 * m[5] + a2 * m[9] + a5 * m[13]);
    o[1] = (a1 * m[1] + a6 * m[9] + a9 * m[13]) - (a0 * m[1] + a7 * m[9] + a8 * m[13]);
    o[2] = (a2 * m[1] + a7 * m[5] + a10 * m[13]) - (a3 * m[1] + a6 * m[5] + a11 * m[13]);
    o[3] = (a5 * m[1] + a8 * m[5] + a11 * m[9]) - (a4 * m[1] + a9 * m[5] + a10 * m[9]);
    const float det = 1.0f / (m[0] * o[0] + m[4] * o[1] + m[8] * o[2] + m[12] * o[3]);
    for (int k = 0; k < 4; ++k) o[k] = det * o[k];
    o[4] = det * ((a1 * m[4] + a2 * m[8] + a5 * m[12]) - (a0 * m[4] + a3 * m[8] + a4 * m[12]));
    o[5] = det * ((a0 * m[0] + a7 * m[8] + a8 * m[12]) - (a1 * m[0] + a6 * m[8] + a9 * m[12]));
    o[6] = det * ((a3 * m[0] + a6 * m[4] + a11 * m[12]) - (a2 * m[0] + a7 * m[4] + a10 * m[12]));
    o[7] = det * ((a4 * m[0] + a9 * m[4] + a10 * m[8]) - (a5 * m[0] + a8 * m[4] + a11 * m[8]));
    o[8] = det * ((b0 * m[7] + b3 * m[11] + b4 * m[15]) - (b1 * m[7] + b2 * m[11] + b5 * m[15]));
    o[9] = det * ((b1 * m[3] + b6 * m[11] + b9 * m[15]) - (b0 * m[3] + b7 * m[11] + b8 * m[15]));
    o[10] = det * ((b2 * m[3] + b7 * m[7] + b10 * m[15]) - (b3 * m[3] + b6 * m[7] + b11 * m[15]));
    o[11] = det * ((b5 * m[3] + b8 * m[7] + b11 * m[11]) - (b4 * m[3] + b9 * m[7] + b10 * m[11]));
    o[12] = det * ((b2 * m[10] + b5 * m[14] + b1 * m[6]) - (b4 * m[14] + b0 * m[6] + b3 * m[10]));
    o[13] = det * ((b8 * m[14] + b0 * m[2] + b7 * m[10]) - (b6 * m[10] + b9 * m[14] + b1 * m[2]));
    o[14] = det * ((b6 * m[6] + b11 * m[14] + b3 * m[2]) - (b10 * m[14] + b2 * m[2] + b7 * m[6]));
    o[15] = det * ((b10 * m[10] + b4 * m[2] + b9 * m[6]) - (b8 * m[6] + b11 * m[10] + b5 * m[2]));
    return o;
}

void half_angle_quat(float ax, float ay, float az, float angle, float q[4]) {
    const float half = 0.5f * angle;
    const float s = std::sin(half), c = std::cos(half);
    q[0] = s * ax;
    q[1] = s * ay;
    q[2] = s * az;
    q[3] = c;
}

}  // namespace

extern "C" int blz_view_setup(BlzCameraViewData* out, float fov, float windowWidth, float windowHeight, float zNear, float zFar,
                              const float position[3], float yaw, float pitch, float pyramidWidth, float pyramidHeight) {
    if (!out || !position || !(windowHeight != 0.0f)) return BLZ_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof *out);
    out->zNear = zNear;
    out->zFar = zFar;
    for (int k = 0; k < 3; ++k) out->position[k] = position[k];

    Mat translation = identity();
    translation[12] = position[0];
    translation[13] = position[1];
    translation[14] = position[2];
    float qYaw[4], qPitch[4];
    half_angle_quat(0.0f, -1.0f, 0.0f, yaw, qYaw);   // yaw about -Y
    half_angle_quat(1.0f, 0.0f, 0.0f, pitch, qPitch);  // pitch about +X
    const Mat rot = multiply(rotation(qYaw[0], qYaw[1], qYaw[2], qYaw[3]), rotation(qPitch[0], qPitch[1], qPitch[2], qPitch[3]));
    const Mat view = inverse(multiply(translation, rot));
    std::memcpy(out->viewMatrix, view.data(), sizeof(float) * 16);

    // infinite far plane, reverse-Z: depth = zNear / z_view
    const float focal = 1.0f / std::tan(fov / 2.0f);
    Mat proj{};
    proj[0] = focal / (windowWidth / windowHeight);
    proj[5] = focal;
    proj[11] = 1.0f;
    proj[14] = zNear;
    out->proj0 = proj[0];
    out->proj5 = proj[5];
    const Mat pv = multiply(proj, view);
    std::memcpy(out->projectionViewMatrix, pv.data(), sizeof(float) * 16);

    // side planes: (row 3 + row 0) and (row 3 + row 1) of the projection, normalised by |xyz|
    float px[4], py[4];
    for (int c = 0; c < 4; ++c) {
        px[c] = proj[4 * c + 3] + proj[4 * c + 0];
        py[c] = proj[4 * c + 3] + proj[4 * c + 1];
    }
    const float nx = std::sqrt(px[0] * px[0] + px[1] * px[1] + px[2] * px[2]);
    const float ny = std::sqrt(py[0] * py[0] + py[1] * py[1] + py[2] * py[2]);
    out->frustumRight = px[0] / nx;
    out->frustumLeft = px[2] / nx;
    out->frustumTop = py[1] / ny;
    out->frustumBottom = py[2] / ny;
    out->lodTarget = (2.0f / out->proj5) * (1.0f / windowHeight);
    out->pyramidWidth = pyramidWidth;
    out->pyramidHeight = pyramidHeight;
    return BLZ_OK;
}
