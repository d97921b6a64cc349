/*
 * Definitions shared by the host builds of the reference's programs
 * (oracle/build_ref.sh): the thread coordinates of the emulated kernels and
 * get_file_lists.  Test infrastructure only.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <filesystem>
#include <regex>
#include <string>
#include <vector>

using namespace std;

dim3 blockIdx, blockDim, threadIdx, gridDim;

/*
 * The reference links get_file_lists from file_lists.cpp, which needs
 * Boost.Filesystem/Regex (absent here).  This is an independent
 * implementation of the behaviour of file_lists.cpp:80-138 with std::
 * facilities: split the base at '/', list regular files of the directory
 * whose name matches ^(base.*)\.ext (regex_search), derive the log / edata /
 * displacement names from capture group 1, and sort each list.
 */
bool get_file_lists(string input, string ext, string tag, vector<string> &dat_files,
                    vector<string> &log_files, vector<string> &disp_files, vector<string> &edat_files) {
    if (input.empty()) return false;
    vector<string> parts;
    string cur;
    for (char c : input) {
        if (c == '/') {
            if (!cur.empty()) parts.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    if (!cur.empty()) parts.push_back(cur);
    if (parts.empty()) return false;
    string base = parts.back();
    string dir;
    if (parts.size() > 1) {
        if (input[0] == '/') dir = "/";
        for (size_t i = 0; i + 1 < parts.size(); ++i) dir += parts[i] + "/";
    } else {
        dir = "./";
    }
    if (base == "*") base = "";
    regex expr("^(" + base + ".*)\\." + ext);
    const string suffix = tag.empty() ? string() : "_" + tag;
    error_code ec;
    if (filesystem::exists(dir, ec)) {
        for (const auto &entry : filesystem::directory_iterator(dir, ec)) {
            if (entry.is_directory()) continue;
            string name = entry.path().filename().string();
            smatch m;
            if (regex_search(name, m, expr)) {
                dat_files.push_back(dir + m[0].str());
                log_files.push_back(dir + m[1].str() + suffix + "_log.txt");
                disp_files.push_back(dir + m[1].str() + suffix);
                edat_files.push_back(dir + m[1].str() + suffix + "_edata.txt");
            }
        }
    }
    sort(dat_files.begin(), dat_files.end());
    sort(log_files.begin(), log_files.end());
    sort(disp_files.begin(), disp_files.end());
    sort(edat_files.begin(), edat_files.end());
    return true;
}

