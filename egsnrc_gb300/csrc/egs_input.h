// Reader for egs++ input files: nested ":start name:" / ":stop name:" blocks
// holding "key = value" lines, '#' comments (the format of
// egs++/egs_input.cpp).  Keys compare case-insensitively with runs of
// blanks collapsed, as in egs++.
#pragma once
#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace egsin {

inline std::string norm(std::string s) {
    std::string o;
    bool sp = false;
    for (char c : s) {
        if (std::isspace((unsigned char)c)) { sp = !o.empty(); continue; }
        if (sp) { o += ' '; sp = false; }
        o += (char)std::tolower((unsigned char)c);
    }
    return o;
}
inline std::string trim(const std::string &s) {
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

struct Item {
    std::string key, value;            // for key = value items
    std::string name;                  // for blocks
    std::vector<std::unique_ptr<Item>> children;
    bool is_block = false;

    const Item *block(const std::string &n) const {
        for (auto &c : children) if (c->is_block && norm(c->name) == norm(n)) return c.get();
        return nullptr;
    }
    std::vector<const Item *> blocks(const std::string &n) const {
        std::vector<const Item *> r;
        for (auto &c : children) if (c->is_block && norm(c->name) == norm(n)) r.push_back(c.get());
        return r;
    }
    bool has(const std::string &k) const {
        for (auto &c : children) if (!c->is_block && norm(c->key) == norm(k)) return true;
        return false;
    }
    std::string get(const std::string &k, const std::string &def = "") const {
        for (auto &c : children) if (!c->is_block && norm(c->key) == norm(k)) return c->value;
        return def;
    }
    std::vector<std::string> all(const std::string &k) const {
        std::vector<std::string> r;
        for (auto &c : children) if (!c->is_block && norm(c->key) == norm(k)) r.push_back(c->value);
        return r;
    }
    static std::vector<std::string> words(const std::string &v) {
        std::string t = v;
        for (char &c : t) if (c == ',' || c == ';') c = ' ';
        std::istringstream is(t);
        std::vector<std::string> w;
        std::string x;
        while (is >> x) w.push_back(x);
        return w;
    }
    static std::vector<double> numbers(const std::string &v) {
        std::vector<double> r;
        for (auto &w : words(v)) r.push_back(std::strtod(w.c_str(), nullptr));
        return r;
    }
    double num(const std::string &k, double def) const {
        if (!has(k)) return def;
        auto v = numbers(get(k));
        return v.empty() ? def : v[0];
    }
};

// Parses a file; returns nullptr and sets err on unbalanced blocks.
inline std::unique_ptr<Item> parse(const std::string &path, std::string &err) {
    std::ifstream f(path);
    if (!f) { err = "cannot open input file " + path; return nullptr; }
    auto root = std::make_unique<Item>();
    root->is_block = true;
    std::vector<Item *> stack{root.get()};
    std::string line;
    int lineno = 0;
    while (std::getline(f, line)) {
        ++lineno;
        size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        line = trim(line);
        if (line.empty()) continue;
        if (line[0] == ':') {
            size_t e = line.find(':', 1);
            if (e == std::string::npos) { err = "malformed block line " + std::to_string(lineno); return nullptr; }
            std::string tag = trim(line.substr(1, e - 1));
            std::string low = norm(tag);
            if (low.rfind("start ", 0) == 0) {
                auto it = std::make_unique<Item>();
                it->is_block = true;
                it->name = trim(tag.substr(6));
                Item *raw = it.get();
                stack.back()->children.push_back(std::move(it));
                stack.push_back(raw);
            } else if (low.rfind("stop ", 0) == 0) {
                if (stack.size() < 2 || norm(stack.back()->name) != norm(tag.substr(5))) {
                    err = "unbalanced :stop " + trim(tag.substr(5)) + ": at line " + std::to_string(lineno);
                    return nullptr;
                }
                stack.pop_back();
            }
            continue;
        }
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        auto it = std::make_unique<Item>();
        it->key = trim(line.substr(0, eq));
        it->value = trim(line.substr(eq + 1));
        stack.back()->children.push_back(std::move(it));
    }
    if (stack.size() != 1) { err = "unterminated block :start " + stack.back()->name + ":"; return nullptr; }
    return root;
}

}  // namespace egsin
