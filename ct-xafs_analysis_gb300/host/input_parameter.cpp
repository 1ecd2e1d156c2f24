// input_parameter.cpp -- parameters of the drop-in CT_reconstruction.
//
// Same keys, value formats and defaults as CT_reconstruction_input_parameter.cpp:40-274 and
// main.cpp:12-47: a line equal to a key is followed by its value -- a whole line for paths
// and names, a stream-extracted number for numeric keys (so a number may sit on the next
// non-empty line).  The key strings are the reference's input format and must match it byte
// for byte.
#include <fstream>
#include <iostream>
#include <sstream>

#include "ct_reconstruction_gb300.hpp"

std::string g_d1 = "input";
std::string g_f1 = "i****.raw";
std::string g_d2 = "output";
std::string g_f2 = "r****.img";
std::string g_f3 = "log.dat";
std::string g_d4 = ".";
std::string g_f4 = "1st.img";
std::string g_d5 = "temp";
int g_fst = 2;
double g_ini = 1;
int g_px = 2048;
int g_pa = 1600;
int g_nx = 2048;
int g_ny = 2048;
int g_ox = 2048;
int g_oy = 2048;
int g_mode = 6;
int g_it = 1;
int g_num = 1;
int g_st = 1;
int g_x = 0;
double g_wt1 = 1.0;
double g_wt2 = 0.01;
int g_ss = 20;
int g_zp = 4096;
std::vector<float> g_ang;
int g_cover = 2;
std::string g_devList = "1";
int numParallel = 10;
int correctionMode = 0;
float amp = 1.0f;
int baseupOrder = 4;
bool CSitBool = false;
float CSlambda = 0.0001f;
int CSoverlap = 1;

std::string ifs_getline(std::istream &is)
{
    std::string s;
    std::getline(is, s);
    if (s.find('\r') != std::string::npos) s.erase(s.end() - 1);
    return s;
}

bool getparameter_inp(const std::string &path)
{
    std::ifstream in(path);
    if (!in) return false;
    std::cout << "Input file found." << std::endl << std::endl;
    while (in.good()) {
        const std::string key = ifs_getline(in);
        if (!in && key.empty()) break;
        if (key == "#Open CL Platform & Device No") g_devList = ifs_getline(in);
        else if (key == "#Number of Parallel processing per one device") in >> numParallel;
        else if (key == "#測定ファイルディレクトリパス") g_d1 = ifs_getline(in);
        else if (key == "#測定ファイル名") g_f1 = ifs_getline(in);
        else if (key == "#出力ファイルディレクトリパス") g_d2 = ifs_getline(in);
        else if (key == "#出力ファイル名") g_f2 = ifs_getline(in);
        else if (key == "#ログファイルパス") g_f3 = ifs_getline(in);
        else if (key == "#初期画像ファイル名") g_f4 = ifs_getline(in);
        else if (key == "#一時ファイルディレクトリパス") g_d5 = ifs_getline(in);
        else if (key == "#レイヤー数") in >> g_num;
        else if (key == "#開始ナンバー") in >> g_st;
        else if (key == "#初期画像の使用 1:Yes 2: No") in >> g_fst;
        else if (key == "#カメラピクセル数") in >> g_px;
        else if (key == "#投影数") in >> g_pa;
        else if (key == "#再構成画像サイズ") {
            in >> g_nx;
            g_ny = g_ox = g_oy = g_nx;
        } else if (key == "#再構成画像サイズ X") in >> g_nx;
        else if (key == "#再構成画像サイズ Y") in >> g_ny;
        else if (key == "#出力画像サイズ X") in >> g_ox;
        else if (key == "#出力画像サイズ Y") in >> g_oy;
        else if (key == "#再構成法") in >> g_mode;
        else if (key == "#反復回数") in >> g_it;
        else if (key == "#AARTファクター") in >> g_wt1;
        else if (key == "#サブセット(OSEM)") in >> g_ss;
        else if (key == "#ゼロパディングサイズ(FBP)") in >> g_zp;
        else if (key == "#投影像補正 0:なし 1: x方向のみ 2:θ方向のみ 3:x,θ方向両方") in >> correctionMode;
        else if (key == "#再構成像強度増幅因子") in >> amp;
        else if (key == "#Base up 減少速度次数 (Hybrid)") in >> baseupOrder;
        else if (key == "#逐次圧縮センシング計算 (FBP適応外)") {
            int v = 0;
            in >> v;
            CSitBool = (v == 1);
        } else if (key == "#逐次圧縮センシング計算加算ファクター") in >> CSlambda;
        else if (key == "#逐次圧縮センシング計算重複レイヤー数") in >> CSoverlap;
    }
    return true;
}

namespace {
// Prompt with the current value in brackets; an empty answer keeps it.
std::string ask(const char *label, const std::string &cur)
{
    std::cout << " " << label << " [" << cur << "] :";
    std::string s;
    std::getline(std::cin, s);
    return s;
}
}  // namespace

void getparameter()
{
    std::string s;
    s = ask("OpenCL device list (ex. 1,2-4)", g_devList);
    if (!s.empty()) g_devList = s;
    s = ask("parallel slices per device", std::to_string(numParallel));
    if (!s.empty()) numParallel = std::stoi(s);
    s = ask("measured file directory", g_d1);
    if (!s.empty()) g_d1 = s;
    s = ask("measured file name", g_f1);
    if (!s.empty()) g_f1 = s;
    s = ask("output directory", g_d2);
    if (!s.empty()) g_d2 = s;
    s = ask("output file name", g_f2);
    if (!s.empty()) g_f2 = s;
    s = ask("log file path", g_f3);
    if (!s.empty()) g_f3 = s;
    s = ask("temporary directory", g_d5);
    if (!s.empty()) g_d5 = s;
    s = ask("number of layers", std::to_string(g_num));
    if (!s.empty()) g_num = std::stoi(s);
    s = ask("start number", std::to_string(g_st));
    if (!s.empty()) g_st = std::stoi(s);
    s = ask("use initial image 1:Yes 2:No", std::to_string(g_fst));
    if (!s.empty()) g_fst = std::stoi(s);
    s = ask("initial image file", g_f4);
    if (!s.empty()) g_f4 = s;
    s = ask("camera pixels", std::to_string(g_px));
    if (!s.empty()) g_px = std::stoi(s);
    s = ask("projections", std::to_string(g_pa));
    if (!s.empty()) g_pa = std::stoi(s);
    s = ask("reconstruction size", std::to_string(g_nx));
    if (!s.empty()) g_nx = g_ny = std::stoi(s);
    s = ask("method 1:AART 2:MART 3:ASIRT 4:MSIRT 5:MLEM 6:OSEM 7:FBP", std::to_string(g_mode));
    if (!s.empty()) g_mode = std::stoi(s);
    s = ask("iterations", std::to_string(g_it));
    if (!s.empty()) g_it = std::stoi(s);
    s = ask("subsets (OSEM)", std::to_string(g_ss));
    if (!s.empty()) g_ss = std::stoi(s);
    s = ask("zero padding (FBP)", std::to_string(g_zp));
    if (!s.empty()) g_zp = std::stoi(s);
    s = ask("projection correction 0:none 1:x 2:theta 3:x,theta", std::to_string(correctionMode));
    if (!s.empty()) correctionMode = std::stoi(s);
}
