// Test infrastructure only: entry point that runs the reference's own
// known-answer tests (tests/test_BackToFrontOrder.cpp,
// tests/test_IndexRangeSplitter.cpp) against the gtest shim in oracle/shims.
#include <gtest/gtest.h>

int main(int argc, char** argv)
{
    testing::InitGoogleTest(&argc, argv);
    return RUN_ALL_TESTS();
}
