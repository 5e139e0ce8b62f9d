// Error convention of the Jet API: every failure throws Jet::Exception whose
// message reads "[file][Line:n][Method:f]: Error in Jet: <message>"
// (reference: include/jet/Abort.hpp:12-97). Tests match on the <message> part.
#pragma once

#include <exception>
#include <sstream>
#include <string>

namespace Jet {

class Exception : public std::exception {
  public:
    explicit Exception(std::string message) noexcept : message_(std::move(message)) {}
    const char *what() const noexcept override { return message_.c_str(); }

  private:
    std::string message_;
};

[[noreturn]] inline void Abort(const char *message, const char *file, int line,
                               const char *function)
{
    std::ostringstream os;
    os << "[" << file << "][Line:" << line << "][Method:" << function
       << "]: Error in Jet: " << message;
    throw Exception(os.str());
}

[[noreturn]] inline void Abort(const std::string &message, const char *file, int line,
                               const char *function)
{
    Abort(message.c_str(), file, line, function);
}

} // namespace Jet

#define JET_ABORT(message) ::Jet::Abort((message), __FILE__, __LINE__, __func__)
#define JET_ABORT_IF(expression, message)                                      \
    do {                                                                       \
        if ((expression))                                                      \
            JET_ABORT(message);                                                \
    } while (0)
#define JET_ABORT_IF_NOT(expression, message)                                  \
    do {                                                                       \
        if (!(expression))                                                     \
            JET_ABORT(message);                                                \
    } while (0)
#define JET_ASSERT(expression)                                                 \
    JET_ABORT_IF_NOT(expression, "Assertion failed: " #expression)
