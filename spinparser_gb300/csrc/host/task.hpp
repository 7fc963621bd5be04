// Task files: parsing, validation and the calculation-status log written back into them.
//
// Restates TaskFileParser (src/TaskFileParser.cpp:21-395) and the ComputationStatus /
// Timestamp helpers it uses (src/SpinParser.hpp, src/lib/Timestamp.hpp): the same element
// and attribute names, the same validation rules and messages, the same discretisations
// (float arithmetic as in the reference), the same status transitions.
#pragma once
#include <ctime>
#include <limits>
#include <map>
#include <string>
#include <utility>
#include <vector>
#include "xml.hpp"

namespace spn {

enum class CalcStatus { New, Running, Postprocessing, Finished };

struct ComputationStatus {
    CalcStatus status = CalcStatus::New;
    std::time_t start_time = 0, checkpoint_time = 0, end_time = 0;
};

// Timestamps as boost::posix_time::to_simple_string writes them ("2020-Jan-31 12:00:00",
// local time) and time_from_string reads them (month as a name or a number).
std::string format_timestamp(std::time_t t);
std::time_t parse_timestamp(const std::string &s);

struct MeasurementSpec {
    std::string name;     // measurement identifier ("correlation")
    std::string output;   // observable file path
    float min_cutoff = 0.0f;
    float max_cutoff = std::numeric_limits<float>::infinity();
    bool defer = false;
    std::vector<std::pair<std::string, std::string>> options;
};

struct Fileset {
    std::string task, obs, data, checkpoint, ldf;
};

// Paths derived from the task file (SpinParser::run, src/SpinParser.cpp:66-70).
Fileset make_fileset(const std::string &task_path);
std::string replace_extension(const std::string &path, const std::string &ext);

struct Task {
    Fileset files;
    XmlNode doc;                      // the parsed document (synthetic root)
    ComputationStatus status;
    std::vector<float> frequencies;   // positive frequencies, ascending
    std::vector<float> cutoffs;       // cutoff values, descending
    std::string lattice;
    int range = 0;
    std::string model;
    std::string symmetry;             // FrgCore identifier ("SU2", "XYZ", "TRI")
    std::map<std::string, std::string> model_options;
    std::vector<MeasurementSpec> measurements;
};

// Parses and validates a task file.  `force_restart` ignores a recorded calculation status
// and removes earlier checkpoint, data and observable files (the reference's --forceRestart);
// without it, a new calculation refuses to overwrite them.  Files are only touched when
// `touch_files` is set (the master rank, src/TaskFileParser.cpp:75-97, 245-259).
Task parse_task(const std::string &task_path, bool force_restart, bool touch_files = true);

// Rewrites the task file with the calculation log of `st` (TaskFileParser::writeTaskFile,
// src/TaskFileParser.cpp:332-355).
void write_task(Task &task, const ComputationStatus &st);

}  // namespace spn
