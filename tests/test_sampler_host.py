"""Host build of the path tracer's sampling code against the reference's
values (no GPU needed)."""
from tests.sampler_check import check_sampler


def test_sampler_host_bitexact(gbrt_lib):
    assert check_sampler(on_device=False) == {}
