// fileio.cpp -- the reference's file formats (CT_reconstruction/fileIO.cpp:11-68) and its
// <base>####<tail> slice naming (GPU.cpp:27-34, :103, :497), plus the device-list syntax of
// OCL_platform_device ("1,2-4", 1-based, share source/OCL_platform_device_class.cpp:55-208).
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>

#include "ct_reconstruction_gb300.hpp"

bool read_log(const std::string &path, int num, std::vector<float> &ang)
{
    std::ifstream in(path);
    if (!in) {
        std::cerr << "file open error [" << path << "]." << std::endl;
        return false;
    }
    ang.assign(num, 0.0f);
    for (int k = 0; k < num; ++k) {  // first token of each line, in degrees
        std::istringstream iss(ifs_getline(in));
        if (!(iss >> ang[k])) {
            // the reference keeps whatever the array held; an angle table shorter than the
            // projection count is an error here
            std::cerr << "angle file [" << path << "]: line " << k + 1 << " holds no angle; " << num
                      << " projections need " << num << " angles." << std::endl;
            return false;
        }
    }
    return true;
}

bool read_data_input(const std::string &dir, const std::string &name, float *buf, size_t count)
{
    const std::string path = dir.empty() ? name : dir + "/" + name;
    std::ifstream in(path, std::ios::in | std::ios::binary);
    if (!in) {
        std::cerr << "file open error [" << name << "]." << std::endl;
        return false;
    }
    in.read(reinterpret_cast<char *>(buf), (std::streamsize)(sizeof(float) * count));
    if ((size_t)in.gcount() != sizeof(float) * count) {
        std::cerr << "short read [" << name << "]: " << in.gcount() << " of " << sizeof(float) * count << " bytes"
                  << std::endl;
        return false;
    }
    return true;
}

bool write_data_output(const std::string &dir, const std::string &name, const float *buf, size_t count)
{
    const std::string path = dir + "/" + name;
    std::ofstream out(path, std::ios::out | std::ios::binary | std::ios::trunc);
    if (!out) {
        std::cerr << "file open error [" << name << "]." << std::endl;
        return false;
    }
    out.write(reinterpret_cast<const char *>(buf), (std::streamsize)(sizeof(float) * count));
    return (bool)out;
}

// g_fst = 1: read the initial image from g_f4; g_fst = 2: uniform g_ini (fileIO.cpp:55-68).
bool first_image(const std::string &path, float *buf, size_t count)
{
    if (g_fst == 1) return read_data_input("", path, buf, count);
    if (g_fst == 2)
        for (size_t i = 0; i < count; ++i) buf[i] = (float)g_ini;
    return true;
}

std::string name_base(const std::string &pattern)
{
    const size_t p = pattern.find_first_of('*');
    return p == std::string::npos ? pattern : pattern.substr(0, p);
}

std::string name_tail(const std::string &pattern)
{
    const size_t p = pattern.find_last_of('*');
    return p == std::string::npos ? std::string() : pattern.substr(p + 1);
}

std::string slice_name(const std::string &pattern, int n)
{
    std::ostringstream os;
    os << name_base(pattern) << std::setfill('0') << std::setw(4) << n << name_tail(pattern);
    return os.str();
}

std::vector<int> parse_device_list(const std::string &list, int ndev)
{
    std::vector<bool> sel(ndev, false);
    std::string s = list;
    int last = 0;
    while (!s.empty()) {
        if (s[0] == ',') {
            s.erase(0, 1);
        } else if (s[0] == '-') {  // last+1 .. end
            s.erase(0, 1);
            size_t used = 0;
            int end = 0;
            try {
                end = std::stoi(s, &used);
            } catch (...) {
                break;
            }
            s.erase(0, used);
            for (int i = last + 1; i <= end; ++i)
                if (i >= 1 && i <= ndev) sel[i - 1] = true;
            last = end;
        } else {
            size_t used = 0;
            int v = 0;
            try {
                v = std::stoi(s, &used);
            } catch (...) {
                break;
            }
            s.erase(0, used);
            if (v >= 1 && v <= ndev) sel[v - 1] = true;
            last = v;
        }
    }
    std::vector<int> out;
    for (int i = 0; i < ndev; ++i)
        if (sel[i]) out.push_back(i);
    return out;
}
