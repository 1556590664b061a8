// STL reader with the reference's interface (GeometryReader.h:9-22):
// Reader::readSTLASCII parses "facet normal / outer loop / vertex x3 /
// endloop / endfacet" blocks and keeps the file's facet normals
// (GeometryReader.cpp:33-117).  An unreadable file prints an error and
// yields no triangles, as in the reference.
#pragma once
#include <string>
#include <vector>

#include "Struct.h"

class Reader {
public:
    std::vector<Triangle> readSTLASCII(const std::string& filename);
};
