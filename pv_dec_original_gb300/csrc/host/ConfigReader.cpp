#include "ConfigReader.h"

#include <cstdlib>
#include <cstring>
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

bool ConfigReader::readEquations(std::vector<std::pair<std::string, std::string>>& equations) {
    std::ifstream file(configFile);
    if (!file.is_open()) {
        error_ = "Error opening file: " + configFile;
        std::cerr << error_ << std::endl;
        return false;
    }
    std::string line, equation, conditions;
    while (std::getline(file, line)) {
        if (line.empty() || line[0] == '#') continue;
        size_t equationPos = line.find("Equation");
        size_t conditionsPos = line.find("Conditions:");
        if (equationPos != std::string::npos) {
            if (!equation.empty() && !conditions.empty()) {
                equations.emplace_back(conditions, equation);
                equation.clear();
                conditions.clear();
            }
        } else if (conditionsPos != std::string::npos) {
            conditions = line.substr(conditionsPos + std::strlen("Conditions:"));
        } else {
            equation += line + '\n';
        }
    }
    if (!equation.empty() && !conditions.empty()) equations.emplace_back(conditions, equation);
    return true;
}

void ConfigReader::printEquations(const std::vector<std::pair<std::string, std::string>>& equations) const {
    for (const auto& eq : equations) std::cout << "Equation Section: " << eq.first << "\n" << eq.second << "\n\n";
}
