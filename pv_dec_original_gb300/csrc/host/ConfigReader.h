// Key/value configuration reader with the reference's interface
// (ConfigReader.h:6-16).  The reference ships the implementation commented
// out (ConfigReader.cpp:9-104); this restates its documented behaviour:
//   - readConfigData: "key value" lines, '#' comments and blank lines
//     skipped, value parsed as a double; a non-numeric value fails the read
//   - readEquations:  "Conditions:" lines open a section whose following
//     lines (up to the next "Equation" marker) form its equation text
// and adds readConfigStrings for non-numeric values (file paths).
#pragma once
#include <map>
#include <string>
#include <utility>
#include <vector>

class ConfigReader {
public:
    explicit ConfigReader(const std::string& configFile);
    bool readConfigData(std::map<std::string, double>& constants);
    bool readConfigStrings(std::map<std::string, std::string>& values);
    bool readEquations(std::vector<std::pair<std::string, std::string>>& equations);
    void printEquations(const std::vector<std::pair<std::string, std::string>>& equations) const;
    const std::string& lastError() const { return error_; }

private:
    std::string configFile;
    std::string error_;
};
