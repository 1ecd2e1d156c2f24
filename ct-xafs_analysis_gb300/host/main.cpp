// main.cpp -- xct_ct_reconstruction: the OS-EM path of CT_reconstruction (main.cpp:54-128)
// on libxct.
//
//   xct_ct_reconstruction [file.inp]          reconstruct (prompts when no .inp is found)
//   xct_ct_reconstruction --print-params f    print the parsed parameters as JSON and exit
//   xct_ct_reconstruction --devlist LIST N    print the devices "1,2-4"-style LIST selects of N
#include <dirent.h>
#include <sys/stat.h>

#include <iostream>
#include <sstream>

#include "ct_reconstruction_gb300.hpp"

namespace {

std::string json_str(const std::string &s)
{
    std::ostringstream o;
    o << '"';
    for (unsigned char c : s) {
        if (c == '"' || c == '\\') o << '\\' << c;
        else if (c < 0x20) o << "\\u00" << "0123456789abcdef"[c >> 4] << "0123456789abcdef"[c & 15];
        else o << c;
    }
    o << '"';
    return o.str();
}

void print_params()
{
    std::cout << "{\"devList\": " << json_str(g_devList) << ", \"numParallel\": " << numParallel
              << ", \"d1\": " << json_str(g_d1) << ", \"f1\": " << json_str(g_f1) << ", \"d2\": " << json_str(g_d2)
              << ", \"f2\": " << json_str(g_f2) << ", \"f3\": " << json_str(g_f3) << ", \"f4\": " << json_str(g_f4)
              << ", \"d5\": " << json_str(g_d5) << ", \"num\": " << g_num << ", \"st\": " << g_st
              << ", \"fst\": " << g_fst << ", \"px\": " << g_px << ", \"pa\": " << g_pa << ", \"nx\": " << g_nx
              << ", \"ny\": " << g_ny << ", \"ox\": " << g_ox << ", \"oy\": " << g_oy << ", \"mode\": " << g_mode
              << ", \"it\": " << g_it << ", \"wt1\": " << g_wt1 << ", \"ss\": " << g_ss << ", \"zp\": " << g_zp
              << ", \"correctionMode\": " << correctionMode << ", \"amp\": " << amp
              << ", \"baseupOrder\": " << baseupOrder << ", \"CSitBool\": " << (CSitBool ? "true" : "false")
              << ", \"CSlambda\": " << CSlambda << ", \"CSoverlap\": " << CSoverlap
              << ", \"first_input\": " << json_str(slice_name(g_f1, g_st))
              << ", \"first_output\": " << json_str(slice_name(g_f2, g_st)) << "}" << std::endl;
}

}  // namespace

int main(int argc, const char *argv[])
{
    if (argc >= 3 && std::string(argv[1]) == "--print-params") {
        if (!getparameter_inp(argv[2])) {
            std::cerr << "Input file not found." << std::endl;
            return 1;
        }
        print_params();
        return 0;
    }
    if (argc >= 4 && std::string(argv[1]) == "--devlist") {
        const std::vector<int> d = parse_device_list(argv[2], std::atoi(argv[3]));
        for (size_t i = 0; i < d.size(); ++i) std::cout << (i ? "," : "") << d[i];
        std::cout << std::endl;
        return 0;
    }

    std::cout << "-----------------------------------------------" << std::endl
              << "    Batch CT reconstruction (OS-EM, GB300 / libxct)" << std::endl
              << "-----------------------------------------------" << std::endl
              << std::endl;
    std::string inp;
    if (argc > 1) {
        inp = argv[1];
    } else {
        std::cout << "Input file path (empty for prompts):" << std::endl;
        std::getline(std::cin, inp);
    }
    if (!getparameter_inp(inp)) {
        std::cout << "Input file not found." << std::endl << "Set the parameters manually." << std::endl << std::endl;
        getparameter();
    }

    // the first sinogram must exist in the input directory (main.cpp:76-108)
    DIR *dir = opendir(g_d1.c_str());
    if (dir == nullptr) {
        std::cout << "Directory not found." << std::endl;
        return 255;
    }
    const std::string first = slice_name(g_f1, g_st);
    bool found = false;
    for (dirent *dp = readdir(dir); dp != nullptr; dp = readdir(dir))
        if (std::string(dp->d_name).find(first) != std::string::npos) {
            std::cout << "raw sinogram file found: " << dp->d_name << std::endl << std::endl;
            found = true;
            break;
        }
    closedir(dir);
    if (!found) {
        std::cout << "No raw file found." << std::endl;
        return 255;
    }

    if (!read_log(g_f3, g_pa, g_ang)) return 1;
    mkdir(g_d2.c_str(), 0755);
    const int rc = GPU();
    return rc == 0 ? 0 : 1;
}
