// TEST INFRASTRUCTURE ONLY.  Stands in for the header src/simulate.cpp
// includes but the reference does not ship (src/simulate.cpp:5).  It
// declares the functions src/simulate.cpp uses before defining them, with
// the reference's own signatures, so its serial core compiles on its own.
#ifndef GLS_REF_SHIM_SIMULATE_H
#define GLS_REF_SHIM_SIMULATE_H
#include <deque>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>
#include "PreProcess.h"

void calc(std::string name, std::vector<VCDBit> input_data, VCDBit &output_data);
void Process(std::map<std::string, TimedValues*> inValues, std::deque<TimedValueSim>& inTimedValues);
void Calculate(std::deque<TimedValueSim> inTimedValues, std::vector<std::string> inputs,
    std::vector<Function> functions, std::vector<Delay> delays, const std::string _out,
    const std::string _out_name, std::unordered_map<std::string, TimedValues*>& _out_value,
    std::map<std::string, TimedValues*> bitValues, VCDTimeUnit time_unit,
    std::vector<std::string> supply1_vec, std::vector<std::string> supply0_vec);
void AddDelay(std::vector<Delay> related_delays, unsigned num_in, int out_sense, VCDTime cur_time,
    std::map<std::string, VCDBit> cur_inValues, std::map<std::string, VCDBit> last_inValues,
    VCDTime &out_time, VCDTimeUnit time_unit);
int CheckDelay(VCDBit pre, VCDBit cur);
void RunFunction(const std::string _out, std::vector<Function> functions,
    std::map<std::string, VCDBit> cur_inValues, VCDBit &cur_out,
    std::vector<std::string> supply1_vec, std::vector<std::string> supply0_vec);
void GetValueAt(std::map<std::string, TimedValues*> bitValues, std::string name, VCDTime time,
    VCDBit &cur, VCDBit &last);
#endif
