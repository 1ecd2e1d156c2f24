// ct_reconstruction_gb300.hpp -- host side of the drop-in CT_reconstruction for the OS-EM
// path, on libxct (include/xct.h) instead of OpenCL.
//
// Same parameters, defaults and file formats as the reference program
// (CT_reconstruction/main.cpp:12-47, CT_reconstruction.hpp:59-135):
//   * parameters come from an .inp file with the reference's "#..." keys
//     (CT_reconstruction_input_parameter.cpp:40-192) or interactively (:194-274);
//   * sinograms are raw float32 [pa][px] files named <base>####<tail> from the '*' pattern of
//     the input file name (GPU.cpp:27-34, :497), the angle log has one angle (degrees) as the
//     first token per line (fileIO.cpp:11-23), reconstructions are raw float32 [oy][ox]
//     (fileIO.cpp:35-43);
//   * OS-EM modes 2 (MART: ss = pa), 4/5 (MSIRT/ML-EM: ss = 1) and 6 (OS-EM: ss = g_ss) run on
//     the GPU through libxct (GPU.cpp:47-80); other modes are not part of this build.
#pragma once
#include <string>
#include <vector>

#include "xct.h"

// ---- parameters (globals of main.cpp:12-47, same defaults) ----
extern std::string g_d1, g_f1, g_d2, g_f2, g_f3, g_d4, g_f4, g_d5;
extern int g_fst;
extern double g_ini;
extern int g_px, g_pa, g_nx, g_ny, g_ox, g_oy, g_mode, g_it, g_num, g_st, g_x;
extern double g_wt1, g_wt2;
extern int g_ss, g_zp, g_cover;
extern std::vector<float> g_ang;
extern std::string g_devList;
extern int numParallel;
extern int correctionMode;
extern float amp;
extern int baseupOrder;
extern bool CSitBool;
extern float CSlambda;
extern int CSoverlap;

// ---- parameters (CT_reconstruction_input_parameter.cpp) ----
// Reads an .inp file; returns false if it cannot be opened (the caller then prompts).
bool getparameter_inp(const std::string &path);
// Interactive prompts with the reference's defaults in brackets (input_parameter.cpp:194-274).
void getparameter();
// One line with a trailing carriage return removed (share source/CTXAFS_analysis_share.cpp:14-27).
std::string ifs_getline(std::istream &is);

// ---- file I/O (fileIO.cpp) ----  All return false on error (the reference exits).
bool read_log(const std::string &path, int num, std::vector<float> &ang);
bool read_data_input(const std::string &dir, const std::string &name, float *buf, size_t count);
bool write_data_output(const std::string &dir, const std::string &name, const float *buf, size_t count);
bool first_image(const std::string &path, float *buf, size_t count);

// ---- devices: "1,2-4" style 1-based list (OCL_platform_device_class.cpp:55-208) ----
std::vector<int> parse_device_list(const std::string &list, int ndev);

// ---- file naming (GPU.cpp:27-34, :103, :497) ----
std::string name_base(const std::string &pattern);
std::string name_tail(const std::string &pattern);
std::string slice_name(const std::string &pattern, int n);

// ---- reconstruction (GPU.cpp:23-97, :562-663) ----
int GPU();
int OSEM_gpu(const std::vector<int> &devices, const std::vector<float> &ang, int ss);
