// pd_flow.hpp - C++ host class over the C ABI, with the method names of the
// reference's PD_flow_opencv (scene_flow_impair.h:53-115) so that code written
// against the reference ports by changing the include and the frame loader.
//
//   PD_flow_opencv                         PD_flow (this file)
//   ctor(rows, i1, i2, z1, z2, out)        ctor(rows)            (no file names: buffers)
//   initializeCUDA()                       initializeCUDA(width, height)
//   loadRGBDFrames()  (PNG via OpenCV)     loadRGBDFrames(i1, z1, i2, z2)  (row-major uint8/uint16)
//   createImagePyramidGPU()  (from I, Z)   createImagePyramidGPU()         (from I, Z)
//   solveSceneFlowGPU()                    solveSceneFlowGPU()
//   dxp, dyp, dzp                          dxp, dyp, dzp  (std::vector<float>, rows*cols, column-major)
//   freeGPUMemory()                        freeGPUMemory()
//
// Errors are reported by exception (pdflow::Error) instead of being ignored.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "pdflow.h"

namespace pdflow {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what)
        : std::runtime_error(what + " failed (" + std::to_string(code) + "): " + pdflow_last_error()), code(code)
    {
    }
    int code;
};

inline void check(int rc, const char* what)
{
    if (rc != PDFLOW_OK) throw Error(rc, what);
}

class PD_flow {
public:
    unsigned rows, cols, width = 0, height = 0, cam_mode = 0, ctf_levels = 0;
    std::vector<float> I, Z;             // staging buffers of the next frame (column-major)
    std::vector<float> dxp, dyp, dzp;    // motion field of the last solve (column-major)
    pdflow_params params;

    explicit PD_flow(unsigned rows_config = 240) : rows(rows_config), cols(rows_config * 320 / 240)
    {
        check(pdflow_default_params(rows, &params), "pdflow_default_params");
        dxp.assign(size_t(rows) * cols, 0.f);
        dyp = dxp;
        dzp = dxp;
    }
    PD_flow(const PD_flow&) = delete;
    PD_flow& operator=(const PD_flow&) = delete;
    ~PD_flow() { freeGPUMemory(); }

    // Image resolution of the camera: 640x480 (cam_mode 1) or 320x240 (cam_mode 2).
    void initializeCUDA(unsigned image_width, unsigned image_height)
    {
        width = image_width;
        height = image_height;
        check(pdflow_create(rows, width, height, &params, &handle_), "pdflow_create");
        unsigned pyr;
        check(pdflow_get_config(handle_, nullptr, nullptr, &ctf_levels, &pyr, &cam_mode), "pdflow_get_config");
        I.assign(size_t(width) * height, 0.f);
        Z = I;
    }

    // Pushes the frame held in I, Z.
    void createImagePyramidGPU() { check(pdflow_push_frame(handle_, I.data(), Z.data()), "pdflow_push_frame"); }

    // Pushes a raw frame (row-major uint8 intensity, uint16 depth = metres*5000).
    void pushRawFrame(const uint8_t* intensity, const uint16_t* depth)
    {
        check(pdflow_push_frame_u16(handle_, intensity, depth), "pdflow_push_frame_u16");
    }

    // Pushes an RGB-D camera frame as the live application reads it (row-major
    // RGB888, uint16 depth in millimetres), converted on the device with that
    // application's arithmetic (PD_flow_mrpt::CaptureFrame); rotate180 stores
    // it in that loop's order.
    void pushCameraFrame(const uint8_t* rgb, const uint16_t* depth_mm, bool rotate180 = true)
    {
        check(pdflow_push_frame_rgb8_mm(handle_, rgb, depth_mm, rotate180 ? 1 : 0), "pdflow_push_frame_rgb8_mm");
    }

    bool loadRGBDFrames(const uint8_t* i1, const uint16_t* z1, const uint8_t* i2, const uint16_t* z2)
    {
        pushRawFrame(i1, z1);
        pushRawFrame(i2, z2);
        return true;
    }

    void solveSceneFlowGPU()
    {
        check(pdflow_solve(handle_), "pdflow_solve");
        check(pdflow_read_flow(handle_, dxp.data(), dyp.data(), dzp.data()), "pdflow_read_flow");
    }

    // CSF_cuda::copyAllSolutions: the motion field and both frames' images at
    // the finest solved level (rows*cols floats each); any pointer may be null.
    void copyAllSolutions(float* dx, float* dy, float* dz, float* depth, float* depth_old, float* colour,
                          float* colour_old, float* xx, float* xx_old, float* yy, float* yy_old)
    {
        check(pdflow_read_all_solutions(handle_, dx, dy, dz, depth, depth_old, colour, colour_old, xx, xx_old, yy,
                                        yy_old),
              "pdflow_read_all_solutions");
    }

    // The live application's per-level copy (scene_flow_visualization.cpp:194-199):
    // keepLevelSolutions(true) before solveSceneFlowGPU records every level;
    // copyAllSolutions(level, ...) then returns solved level `level` (0 = the
    // coarsest) with that level's pyramid images.
    void keepLevelSolutions(bool keep)
    {
        check(pdflow_keep_level_solutions(handle_, keep ? 1 : 0), "pdflow_keep_level_solutions");
    }
    void copyAllSolutions(unsigned level, float* dx, float* dy, float* dz, float* depth, float* depth_old,
                          float* colour, float* colour_old, float* xx, float* xx_old, float* yy, float* yy_old)
    {
        check(pdflow_read_level_solutions(handle_, level, dx, dy, dz, depth, depth_old, colour, colour_old, xx,
                                          xx_old, yy, yy_old),
              "pdflow_read_level_solutions");
    }

    void freeGPUMemory()
    {
        if (handle_) pdflow_destroy(handle_);
        handle_ = nullptr;
    }

    pdflow_solver* handle() const { return handle_; }

private:
    pdflow_solver* handle_ = nullptr;
};

}  // namespace pdflow
