// ref_levels_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own levelization -- GenerateAdjacencyList,
// SetInDegrees and TopologyOrder of src/process.cpp:90-176, extracted from
// the reference sources by oracle/build.py -- on an instance list, the way
// the reference's `process` calls them (src/process.cpp:226-247).
//
// input (text): n, then per instance: name, n_out, its output nets, n_in,
// its input nets.  output: one line per level, the instance ids in order.
//
// usage: ref_levels <instances.txt>
#include <cstdio>
#include <fstream>
#include <map>
#include <string>
#include <vector>
#include "Instance.h"

using std::string;

void GenerateAdjacencyList(std::map<std::string, Instance> &instances, std::vector<string> &inst_names,
                           std::map<std::string, std::vector<int>> net_instance_map, std::vector<int> &adjacencyList,
                           std::vector<int> &edgesOffset, std::vector<int> &edgesSize);
void SetInDegrees(std::vector<int> adjacencyList, std::vector<int> edgesOffset, std::vector<int> edgesSize,
                  std::vector<int> &indegrees);
std::vector<std::vector<int>> TopologyOrder(std::vector<int> adjacencyList, std::vector<int> edgesOffset,
                                            std::vector<int> edgesSize, std::vector<int> indegrees, int flag,
                                            std::vector<std::vector<int>> levels, int n);

int main(int argc, char **argv)
{
    if (argc != 2) {
        fprintf(stderr, "usage: ref_levels <instances.txt>\n");
        return 2;
    }
    std::ifstream f(argv[1]);
    size_t n = 0;
    f >> n;
    std::map<std::string, Instance> instances;
    std::vector<string> names;
    std::map<std::string, std::vector<int>> net_instance_map;   // net -> readers, as parse_gv builds it
    for (size_t i = 0; i < n && f; ++i) {
        string name;
        size_t no = 0, ni = 0;
        f >> name >> no;
        Instance in;
        in.name = name;
        for (size_t k = 0; k < no; ++k) {
            string net;
            f >> net;
            in.set_out("o" + std::to_string(k), net);
            in.out_net.push_back(net);
        }
        f >> ni;
        for (size_t k = 0; k < ni; ++k) {
            string net;
            f >> net;
            in.set_in("i" + std::to_string(k), net);
            in.in_net.push_back(net);
            net_instance_map[net].push_back((int)i);
        }
        names.push_back(name);
        instances.insert(std::make_pair(name, in));
    }
    if (!f) {
        fprintf(stderr, "ref_levels: malformed input\n");
        return 2;
    }
    std::vector<int> adjacency, offset, size;
    GenerateAdjacencyList(instances, names, net_instance_map, adjacency, offset, size);
    std::vector<int> indegrees(offset.size());
    SetInDegrees(adjacency, offset, size, indegrees);
    std::vector<std::vector<int>> none;
    const std::vector<std::vector<int>> levels = TopologyOrder(adjacency, offset, size, indegrees, 1, none,
                                                               (int)offset.size());
    for (auto &lv : levels) {
        for (size_t k = 0; k < lv.size(); ++k) printf(k ? " %d" : "%d", lv[k]);
        printf("\n");
    }
    return 0;
}
