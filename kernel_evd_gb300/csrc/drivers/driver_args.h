// Run-time overrides of the stage drivers' compile-time configuration.
//
// With no arguments a driver runs exactly as the reference's program does, with
// its constants (the -D defaults).  Optional overrides, in any order:
//   --key value | --key=value     one setting (keys: the driver's table)
//   --config file.json            a flat JSON object of settings, e.g.
//                                 {"ndata": 2000, "mgrid": 8, "precision": "fp64"}
//   --print-config                print the resolved settings and the file names,
//                                 touch no file and no GPU, exit 0
//   --help                        list the settings and their defaults
// Settings given on the command line win over the JSON file wherever they
// appear.  An unknown key, a malformed value or a bad JSON file ends the program
// with status 2 before any work, as a misconfigured reference program would fail
// to compile.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

struct DriverSetting {
    const char* key;
    double value;
    enum Kind { kInt, kReal, kPrecision, kFlag } kind;
    const char* help;
};

class DriverConfig {
  public:
    DriverConfig(const char* prog, std::vector<DriverSetting> s) : prog_(prog), s_(std::move(s)) {}

    void parse(int argc, char** argv) {
        std::vector<std::pair<std::string, std::string>> cli;
        std::string json;
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            if (a == "--help" || a == "-h") {
                usage(stdout);
                exit(0);
            }
            if (a == "--print-config") {
                print_only = true;
                continue;
            }
            if (a.rfind("--", 0) != 0) die("unexpected argument " + a);
            a = a.substr(2);
            std::string key = a, val;
            const size_t eq = a.find('=');
            if (eq != std::string::npos) {
                key = a.substr(0, eq);
                val = a.substr(eq + 1);
            } else {
                if (i + 1 >= argc) die("--" + key + " needs a value");
                val = argv[++i];
            }
            if (key == "config") json = val;
            else cli.push_back({key, val});
        }
        if (!json.empty()) read_json(json);
        for (const auto& kv : cli) set(kv.first, kv.second);
    }

    double get(const char* key) const {
        for (const auto& s : s_)
            if (!strcmp(s.key, key)) return s.value;
        fprintf(stderr, "%s: internal: no setting %s\n", prog_, key);
        exit(2);
    }
    size_t size(const char* key) const { return (size_t)get(key); }
    int integer(const char* key) const { return (int)get(key); }

    void print(FILE* f) const {
        for (const auto& s : s_) {
            if (s.kind == DriverSetting::kPrecision) fprintf(f, "%s = %s\n", s.key, s.value == 0 ? "fp64" : "mixed");
            else if (s.kind == DriverSetting::kReal) fprintf(f, "%s = %.17g\n", s.key, s.value);
            else fprintf(f, "%s = %lld\n", s.key, (long long)s.value);
        }
    }

    bool print_only = false;

  private:
    [[noreturn]] void die(const std::string& msg) const {
        fprintf(stderr, "%s: %s\n", prog_, msg.c_str());
        usage(stderr);
        exit(2);
    }

    void usage(FILE* f) const {
        fprintf(f, "usage: %s [--key value ...] [--config file.json] [--print-config]\n", prog_);
        for (const auto& s : s_) {
            if (s.kind == DriverSetting::kPrecision)
                fprintf(f, "  --%-10s %s (default %s)\n", s.key, s.help, s.value == 0 ? "fp64" : "mixed");
            else
                fprintf(f, "  --%-10s %s (default %.17g)\n", s.key, s.help, s.value);
        }
    }

    void set(const std::string& key, const std::string& val) {
        for (auto& s : s_) {
            if (key != s.key) continue;
            if (s.kind == DriverSetting::kPrecision) {
                if (val == "fp64" || val == "0") s.value = 0;
                else if (val == "mixed" || val == "1") s.value = 1;
                else die("--" + key + ": fp64 or mixed, not " + val);
                return;
            }
            if (s.kind == DriverSetting::kFlag && (val == "true" || val == "false")) {
                s.value = val == "true";
                return;
            }
            char* end = nullptr;
            const double v = strtod(val.c_str(), &end);
            if (val.empty() || *end != 0 || !(v == v)) die("--" + key + ": not a number: " + val);
            if (s.kind != DriverSetting::kReal && (v < 0 || v != (double)(long long)v))
                die("--" + key + ": not a nonnegative integer: " + val);
            if (s.kind == DriverSetting::kFlag && v > 1) die("--" + key + ": 0 or 1, not " + val);
            s.value = v;
            return;
        }
        die("unknown setting --" + key);
    }

    // A flat JSON object whose values are numbers, strings or true/false.
    void read_json(const std::string& path) {
        FILE* f = fopen(path.c_str(), "rb");
        if (!f) die("cannot open " + path);
        std::string t;
        char buf[4096];
        size_t n;
        while ((n = fread(buf, 1, sizeof(buf), f)) > 0) t.append(buf, n);
        fclose(f);
        size_t p = 0;
        auto ws = [&]() {
            while (p < t.size() && (t[p] == ' ' || t[p] == '\t' || t[p] == '\n' || t[p] == '\r')) ++p;
        };
        auto str = [&]() {
            if (p >= t.size() || t[p] != '"') die(path + ": expected a string at byte " + std::to_string(p));
            std::string s;
            for (++p; p < t.size() && t[p] != '"'; ++p) {
                if (t[p] == '\\') die(path + ": escapes are not supported");
                s += t[p];
            }
            if (p >= t.size()) die(path + ": unterminated string");
            ++p;
            return s;
        };
        ws();
        if (p >= t.size() || t[p] != '{') die(path + ": expected a JSON object");
        ++p;
        ws();
        if (p < t.size() && t[p] == '}') {
            ++p;
        } else {
            for (;;) {
                ws();
                const std::string key = str();
                ws();
                if (p >= t.size() || t[p] != ':') die(path + ": expected ':' after \"" + key + "\"");
                ++p;
                ws();
                std::string val;
                if (p < t.size() && t[p] == '"') {
                    val = str();
                } else {
                    const size_t q = p;
                    while (p < t.size() && t[p] != ',' && t[p] != '}' && t[p] != ' ' && t[p] != '\n' &&
                           t[p] != '\t' && t[p] != '\r')
                        ++p;
                    val = t.substr(q, p - q);
                }
                set(key, val);
                ws();
                if (p < t.size() && t[p] == ',') {
                    ++p;
                    continue;
                }
                if (p < t.size() && t[p] == '}') {
                    ++p;
                    break;
                }
                die(path + ": expected ',' or '}' at byte " + std::to_string(p));
            }
        }
        ws();
        if (p != t.size()) die(path + ": trailing text after the object");
    }

    const char* prog_;
    std::vector<DriverSetting> s_;
};
