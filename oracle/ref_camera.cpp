// ref_camera.cpp — TEST INFRASTRUCTURE. Links the reference's own camera code (compiled from the
// reference tree by oracle/ref_build.py, never copied) and exposes it with C linkage so the tests
// can compare its CameraViewData bytes with blz_view_setup and the oracle.
#include "Game/blitCamera.h"

extern "C" void ref_view_setup(void* out256, float fov, float w, float h, float zNear, float zFar, const float* pos,
                               float yaw, float pitch, float pw, float ph)
{
    static BlitzenEngine::Camera cam;  // large; keep off the stack
    BlitzenEngine::SetupCamera(cam, fov, w, h, zNear, BlitML::vec3{pos[0], pos[1], pos[2]}, zFar, yaw, pitch);
    cam.viewData.pyramidWidth = pw;
    cam.viewData.pyramidHeight = ph;
    static_assert(sizeof(cam.viewData) == 256, "CameraViewData is 256 bytes");
    __builtin_memcpy(out256, &cam.viewData, 256);
}
