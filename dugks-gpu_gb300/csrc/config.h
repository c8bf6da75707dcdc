// config.txt reader with the reference's semantics (src/config.h:17-74):
//   * lines split at '='; a line without '=' is ignored (how '#' comments work)
//   * key = text before the first '=', value = text up to the next '=' (or end)
//   * no whitespace trimming; the first occurrence of a key wins (map::insert)
//   * integers parse like std::stoi, reals like std::stof (strtof, i.e. float
//     precision, then widened) -- src/numerics.cu:74-99.
// Unlike the reference a missing or unparsable key is an error status, not an
// uncaught exception.
#pragma once
#include <map>
#include <string>

namespace dg {

class ConfigFile {
public:
    bool load_file(const std::string &path, std::string &err);
    void load_text(const std::string &text);
    bool has(const std::string &key) const { return kv_.count(key) != 0; }
    // required keys
    bool get_int(const std::string &key, int &out, std::string &err) const;
    bool get_float(const std::string &key, double &out, std::string &err) const;  // std::stof then widen
    bool get_string(const std::string &key, std::string &out, std::string &err) const;
    // optional keys (extensions of this engine); default when absent
    bool opt_int(const std::string &key, int def, int &out, std::string &err) const;
    bool opt_float(const std::string &key, double def, double &out, std::string &err) const;
    bool opt_double(const std::string &key, double def, double &out, std::string &err) const;  // strtod precision
    std::string opt_string(const std::string &key, const std::string &def) const;

private:
    std::map<std::string, std::string> kv_;
};

// std::stoi / std::stof equivalents returning false instead of throwing
bool parse_stoi(const std::string &s, int &out);
bool parse_stof(const std::string &s, float &out);
bool parse_stod(const std::string &s, double &out);

}  // namespace dg
