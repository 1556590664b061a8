#include "ConfigReader.h"

#include <cstdlib>
#include <fstream>
#include <iostream>

ConfigReader::ConfigReader(const std::string& f) : configFile(f) {}

namespace {

bool split_line(const std::string& line, std::string& key, std::string& value) {
    size_t pos = line.find_first_of(" \t");
    if (pos == std::string::npos) return false;
    key = line.substr(0, pos);
    size_t v = line.find_first_not_of(" \t", pos);
    value = v == std::string::npos ? std::string() : line.substr(v);
    while (!value.empty() && (value.back() == '\r' || value.back() == ' ' || value.back() == '\t')) value.pop_back();
    return true;
}

}  // namespace

bool ConfigReader::readConfigData(std::map<std::string, double>& configData) {
    std::ifstream file(configFile);
    if (!file.is_open()) {
        error_ = "Error opening file: " + configFile;
        std::cerr << error_ << std::endl;
        return false;
    }
    std::string line;
    while (std::getline(file, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::string key, value;
        if (!split_line(line, key, value)) continue;
        const char* s = value.c_str();
        char* end = nullptr;
        double d = std::strtod(s, &end);
        if (end == s) {
            error_ = "Error converting value to double for key " + key;
            std::cerr << error_ << std::endl;
            return false;
        }
        configData[key] = d;
    }
    return true;
}

bool ConfigReader::readConfigStrings(std::map<std::string, std::string>& values) {
    std::ifstream file(configFile);
    if (!file.is_open()) {
        error_ = "Error opening file: " + configFile;
        return false;
    }
    std::string line;
    while (std::getline(file, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::string key, value;
        if (split_line(line, key, value)) values[key] = value;
    }
    return true;
}

// Equation blocks.  Grammar (comment and blank lines are skipped):
//   marker    := any line containing the word "Equation"
//   condition := any other line containing "Conditions:"; the text after
//                the tag is the block's condition (a later one replaces it)
//   body      := every other line, appended with its newline
// A marker closes the open block when it has both a condition and a body
// (an incomplete block stays open and keeps collecting); the end of the
// file closes it the same way.  Blocks come out as (condition, body).
namespace {

struct EquationBlock {
    std::string condition, body;
    bool complete() const { return !condition.empty() && !body.empty(); }
};

}  // namespace

bool ConfigReader::readEquations(std::vector<std::pair<std::string, std::string>>& equations) {
    std::ifstream in(configFile);
    if (!in) {
        error_ = "Error opening file: " + configFile;
        std::cerr << error_ << std::endl;
        return false;
    }
    static const char kTag[] = "Conditions:";
    EquationBlock open;
    auto close_if_complete = [&]() {
        if (!open.complete()) return;
        equations.emplace_back(std::move(open.condition), std::move(open.body));
        open = EquationBlock{};
    };
    for (std::string text; std::getline(in, text);) {
        if (text.empty() || text.front() == '#') continue;
        if (text.find("Equation") != std::string::npos) {
            close_if_complete();
            continue;
        }
        const size_t tag = text.find(kTag);
        if (tag != std::string::npos) open.condition = text.substr(tag + sizeof(kTag) - 1);
        else open.body.append(text).push_back('\n');
    }
    close_if_complete();
    return true;
}

void ConfigReader::printEquations(const std::vector<std::pair<std::string, std::string>>& equations) const {
    for (size_t k = 0; k < equations.size(); ++k)
        std::cout << "Equation Section: " << equations[k].first << '\n' << equations[k].second << "\n\n";
}
