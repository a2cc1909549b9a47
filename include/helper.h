/*
 * helper.h - the reference's timing helper (helper.h: ppf::Timer): a scope timer that
 * prints "<label> cost(ms): <elapsed>" when released or destroyed.
 */
#pragma once

#include <chrono>
#include <iostream>
#include <string>
#include <utility>

namespace ppf {

class Timer {
public:
    explicit Timer(std::string content)
        : content_(std::move(content)), start_(std::chrono::steady_clock::now()) {}
    ~Timer() {
        if (!released_)
            release();
    }
    void release() {
        released_ = true;
        const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
                            std::chrono::steady_clock::now() - start_)
                            .count();
        std::cout << content_ << " cost(ms): " << ms << std::endl;
    }

private:
    std::string                           content_;
    std::chrono::steady_clock::time_point start_;
    bool                                  released_ = false;
};

} // namespace ppf
