// Entry point with the reference's shape (reference: prover.cpp:23-37): runs
// the tight-rectangle proof, then the size-bound proof, on the GB300 through
// the drop-in drivers.  argv is ignored, as in the reference.
namespace circlecover {
namespace rectangle_size_bound {
void find_critical_intervals();
}
namespace tight_rectangle {
void find_critical_intervals();
}
}  // namespace circlecover

int main(int, const char*[]) {
    circlecover::tight_rectangle::find_critical_intervals();
    circlecover::rectangle_size_bound::find_critical_intervals();
    return 0;
}
