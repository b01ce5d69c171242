from .structured import JsonlLogger, close_all_jsonl_logs

__all__ = ["JsonlLogger", "close_all_jsonl_logs"]
