#include "config.h"

#include <cerrno>
#include <climits>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace dg {

void ConfigFile::load_text(const std::string &text)
{
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line, '\n')) {
        const std::string::size_type a = line.find('=');
        if (a == std::string::npos) continue;
        const std::string::size_type b = line.find('=', a + 1);
        const std::string key = line.substr(0, a);
        const std::string val = b == std::string::npos ? line.substr(a + 1) : line.substr(a + 1, b - a - 1);
        kv_.insert({key, val});  // first occurrence wins
    }
}

bool ConfigFile::load_file(const std::string &path, std::string &err)
{
    std::ifstream f(path);
    if (!f) {
        err = "cannot open config file '" + path + "'";
        return false;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    load_text(ss.str());
    return true;
}

bool parse_stoi(const std::string &s, int &out)
{
    const char *p = s.c_str();
    char *end = nullptr;
    errno = 0;
    const long v = std::strtol(p, &end, 10);
    if (end == p) return false;
    if (errno == ERANGE || v < INT_MIN || v > INT_MAX) return false;
    out = int(v);
    return true;
}

bool parse_stof(const std::string &s, float &out)
{
    const char *p = s.c_str();
    char *end = nullptr;
    errno = 0;
    const float v = std::strtof(p, &end);
    if (end == p) return false;
    if (errno == ERANGE) return false;
    out = v;
    return true;
}

bool parse_stod(const std::string &s, double &out)
{
    const char *p = s.c_str();
    char *end = nullptr;
    errno = 0;
    const double v = std::strtod(p, &end);
    if (end == p) return false;
    if (errno == ERANGE) return false;
    out = v;
    return true;
}

bool ConfigFile::get_string(const std::string &key, std::string &out, std::string &err) const
{
    auto it = kv_.find(key);
    if (it == kv_.end()) {
        err = "config key not found: " + key;
        return false;
    }
    out = it->second;
    return true;
}

bool ConfigFile::get_int(const std::string &key, int &out, std::string &err) const
{
    std::string s;
    if (!get_string(key, s, err)) return false;
    if (!parse_stoi(s, out)) {
        err = "config key '" + key + "': not an integer: '" + s + "'";
        return false;
    }
    return true;
}

bool ConfigFile::get_float(const std::string &key, double &out, std::string &err) const
{
    std::string s;
    if (!get_string(key, s, err)) return false;
    float f = 0;
    if (!parse_stof(s, f)) {
        err = "config key '" + key + "': not a real number: '" + s + "'";
        return false;
    }
    out = double(f);
    return true;
}

bool ConfigFile::opt_int(const std::string &key, int def, int &out, std::string &err) const
{
    if (!has(key)) {
        out = def;
        return true;
    }
    return get_int(key, out, err);
}

bool ConfigFile::opt_float(const std::string &key, double def, double &out, std::string &err) const
{
    if (!has(key)) {
        out = def;
        return true;
    }
    return get_float(key, out, err);
}

bool ConfigFile::opt_double(const std::string &key, double def, double &out, std::string &err) const
{
    if (!has(key)) {
        out = def;
        return true;
    }
    std::string s;
    if (!get_string(key, s, err)) return false;
    if (!parse_stod(s, out)) {
        err = "config key '" + key + "': not a real number: '" + s + "'";
        return false;
    }
    return true;
}

std::string ConfigFile::opt_string(const std::string &key, const std::string &def) const
{
    auto it = kv_.find(key);
    return it == kv_.end() ? def : it->second;
}

}  // namespace dg
